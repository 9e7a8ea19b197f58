// Launcher for the reference's own GPU kernels (MRCuda/MRCudaFastWindingNumber.cu), built from the
// reference sources into oracle/_ref/ by oracle/ref/build_ref.py.
//
// TEST / BENCH INFRASTRUCTURE ONLY: it lets the parity tests compare the library with the
// reference's GPU path and lets the benchmark time that path ("plain MRCuda") on the same GPU.
// The product never loads it.
//
// The kernels are loaded with the CUDA driver API (libcuda is opened at run time, so this file
// links against nothing) and launched with the reference's grid shape: one thread per query, 32
// threads per block (MRCudaFastWindingNumber.cu:15 and :245-274).  Arguments follow the kernel
// signatures (.cu:135-243) and the reference's by-value layouts:
//   int3 dims; Matrix4 {float3 x, y, z, b; bool isIdentity} (MRCuda/MRCudaMath.cuh:157-163);
//   DistanceToMeshOptions {float minDistSq, maxDistSq; bool nullOutsideMinMax;
//                          float windingNumberThreshold, windingNumberBeta}
//   (MRMesh/MRDistanceToMeshOptions.h:10-33);
//   Dipole {float3 pos; float area; float3 dirArea; float rr} (MRCudaFastWindingNumber.cuh:16-22);
//   Node3 {Box3 {float3 min, max}; int l, r} (MRCudaMath.cuh:101-104);
//   meshPoints float3[]; FaceToThreeVerts {int verts[3]} (MRCudaMath.cuh:120-123).
#include <cuda.h>
#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace {

struct Int3 {
    int x, y, z;
};
struct Matrix4 {
    float m[12];  // rows x, y, z, then b
    bool isIdentity;
};
static_assert(sizeof(Matrix4) == 52, "Matrix4 layout");
struct Options {
    float minDistSq, maxDistSq;
    bool nullOutsideMinMax;
    float windingNumberThreshold, windingNumberBeta;
};
static_assert(sizeof(Options) == 20, "DistanceToMeshOptions layout");

using PInit = CUresult (*)(unsigned);
using PCtxGetCurrent = CUresult (*)(CUcontext*);
using PCtxSetCurrent = CUresult (*)(CUcontext);
using PDeviceGet = CUresult (*)(CUdevice*, int);
using PPrimaryRetain = CUresult (*)(CUcontext*, CUdevice);
using PModuleLoad = CUresult (*)(CUmodule*, const char*);
using PModuleGetFunction = CUresult (*)(CUfunction*, CUmodule, const char*);
using PLaunch = CUresult (*)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, CUstream,
                             void**, void**);
using PErrorString = CUresult (*)(CUresult, const char**);

struct Driver {
    void* so = nullptr;
    PInit init = nullptr;
    PCtxGetCurrent ctxGetCurrent = nullptr;
    PCtxSetCurrent ctxSetCurrent = nullptr;
    PDeviceGet deviceGet = nullptr;
    PPrimaryRetain primaryRetain = nullptr;
    PModuleLoad moduleLoad = nullptr;
    PModuleGetFunction getFunction = nullptr;
    PLaunch launch = nullptr;
    PErrorString errorString = nullptr;
    CUmodule module = nullptr, projModule = nullptr;
    CUfunction sdf = nullptr, grid = nullptr, vec = nullptr, mesh = nullptr, proj = nullptr;
};

Driver g;
std::mutex g_mu;
char g_err[512] = "";

// mangled names of the four kernels (namespace MR::Cuda)
const char* kSdf =
    "_ZN2MR4Cuda20signedDistanceKernelE4int3NS0_7Matrix4EPKNS0_6DipoleEPKNS0_5Node3EPK6float3PKNS0_16FaceToThreeVertsEPfNS_"
    "21DistanceToMeshOptionsEmm";
const char* kGrid =
    "_ZN2MR4Cuda31fastWindingNumberFromGridKernelE4int3NS0_7Matrix4EPKNS0_6DipoleEPKNS0_5Node3EPK6float3PKNS0_"
    "16FaceToThreeVertsEPffmm";
const char* kMesh =
    "_ZN2MR4Cuda31fastWindingNumberFromMeshKernelEPKNS0_6DipoleEPKNS0_5Node3EPK6float3PKNS0_16FaceToThreeVertsEPffmm";
const char* kVec =
    "_ZN2MR4Cuda33fastWindingNumberFromVectorKernelEPK6float3PKNS0_6DipoleEPKNS0_5Node3ES3_PKNS0_16FaceToThreeVertsEPffim";

// MRCuda/MRCudaPointsToMeshProjector.cu:6-111 (launched with 640 threads per block, .cu:113-120)
const char* kProj =
    "_ZN2MR4Cuda6kernelEPK6float3PKNS0_5Node3ES3_PKNS0_16FaceToThreeVertsEPNS0_20MeshProjectionResultENS0_7Matrix4ESC_ffm";

Matrix4 matrix(const float* xf) {  // NULL -> Matrix4{} (identity flag set)
    Matrix4 m{};
    if (xf) {
        std::memcpy(m.m, xf, sizeof(m.m));
        m.isIdentity = false;
    } else {
        const float id[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
        std::memcpy(m.m, id, sizeof(id));
        m.isIdentity = true;
    }
    return m;
}

int fail(const char* what, CUresult r) {
    const char* s = nullptr;
    if (g.errorString) g.errorString(r, &s);
    std::snprintf(g_err, sizeof(g_err), "%s: CUDA driver error %d (%s)", what, int(r), s ? s : "?");
    return int(r) ? int(r) : -1;
}

template <class T> bool sym(T& f, const char* name) {
    f = reinterpret_cast<T>(dlsym(g.so, name));
    if (!f) std::snprintf(g_err, sizeof(g_err), "libcuda has no %s", name);
    return f != nullptr;
}

unsigned blocks(uint64_t n) { return unsigned((n + 31) / 32); }

}  // namespace

extern "C" {

const char* mrc_last_error() { return g_err; }

// Loads the reference kernels (cubin, else PTX) into the current context (the primary context of
// `device` when none is current).  Returns 0 on success.
int mrc_load(const char* cubin, const char* ptx, int device) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g.module) return 0;
    if (!g.so) {
        g.so = dlopen("libcuda.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!g.so) {
            std::snprintf(g_err, sizeof(g_err), "cannot open libcuda.so.1");
            return -1;
        }
    }
    if (!sym(g.init, "cuInit") || !sym(g.ctxGetCurrent, "cuCtxGetCurrent") || !sym(g.ctxSetCurrent, "cuCtxSetCurrent") ||
        !sym(g.deviceGet, "cuDeviceGet") || !sym(g.primaryRetain, "cuDevicePrimaryCtxRetain") ||
        !sym(g.moduleLoad, "cuModuleLoad") || !sym(g.getFunction, "cuModuleGetFunction") ||
        !sym(g.launch, "cuLaunchKernel") || !sym(g.errorString, "cuGetErrorString"))
        return -1;
    CUresult r = g.init(0);
    if (r) return fail("cuInit", r);
    CUcontext ctx = nullptr;
    if ((r = g.ctxGetCurrent(&ctx))) return fail("cuCtxGetCurrent", r);
    if (!ctx) {
        CUdevice dev;
        if ((r = g.deviceGet(&dev, device))) return fail("cuDeviceGet", r);
        if ((r = g.primaryRetain(&ctx, dev))) return fail("cuDevicePrimaryCtxRetain", r);
        if ((r = g.ctxSetCurrent(ctx))) return fail("cuCtxSetCurrent", r);
    }
    CUmodule m = nullptr;
    r = cubin && *cubin ? g.moduleLoad(&m, cubin) : CUDA_ERROR_FILE_NOT_FOUND;
    if (r && ptx && *ptx) r = g.moduleLoad(&m, ptx);
    if (r) return fail("cuModuleLoad (reference kernels)", r);
    if ((r = g.getFunction(&g.sdf, m, kSdf))) return fail("signedDistanceKernel", r);
    if ((r = g.getFunction(&g.grid, m, kGrid))) return fail("fastWindingNumberFromGridKernel", r);
    if ((r = g.getFunction(&g.vec, m, kVec))) return fail("fastWindingNumberFromVectorKernel", r);
    if ((r = g.getFunction(&g.mesh, m, kMesh))) return fail("fastWindingNumberFromMeshKernel", r);
    g.module = m;
    return 0;
}

// signedDistanceKernel over grid indices [chunkOffset, chunkOffset + chunkSize); out is
// chunk-relative.  xf = 12 floats (rows of A, then b); identity selects Matrix4{} as the reference
// does for an identity transform (MRCudaMath.cpp:19-31).
int mrc_signed_distance(const int32_t dims[3], const float xf[12], int identity, const void* dipoles, const void* nodes,
                        const void* points, const void* faces, float* out, float minDistSq, float maxDistSq,
                        int nullOutsideMinMax, float threshold, float beta, uint64_t chunkSize, uint64_t chunkOffset,
                        void* stream) {
    if (!g.module) return -1;
    if (chunkSize == 0) return 0;  // the kernels reject an empty launch
    Int3 d{dims[0], dims[1], dims[2]};
    Matrix4 m{};
    if (identity) {
        const float id[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
        std::memcpy(m.m, id, sizeof(id));
        m.isIdentity = true;
    } else {
        std::memcpy(m.m, xf, sizeof(m.m));
        m.isIdentity = false;
    }
    Options o{minDistSq, maxDistSq, nullOutsideMinMax != 0, threshold, beta};
    size_t cs = chunkSize, co = chunkOffset;
    void* args[] = {&d, &m, &dipoles, &nodes, &points, &faces, &out, &o, &cs, &co};
    const CUresult r = g.launch(g.sdf, blocks(chunkSize), 1, 1, 32, 1, 1, 0, CUstream(stream), args, nullptr);
    return r ? fail("signedDistanceKernel launch", r) : 0;
}

int mrc_from_grid(const int32_t dims[3], const float xf[12], int identity, const void* dipoles, const void* nodes,
                  const void* points, const void* faces, float* out, float beta, uint64_t chunkSize, uint64_t chunkOffset,
                  void* stream) {
    if (!g.module) return -1;
    if (chunkSize == 0) return 0;  // the kernels reject an empty launch
    Int3 d{dims[0], dims[1], dims[2]};
    Matrix4 m{};
    if (identity) {
        const float id[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
        std::memcpy(m.m, id, sizeof(id));
        m.isIdentity = true;
    } else {
        std::memcpy(m.m, xf, sizeof(m.m));
        m.isIdentity = false;
    }
    size_t cs = chunkSize, co = chunkOffset;
    void* args[] = {&d, &m, &dipoles, &nodes, &points, &faces, &out, &beta, &cs, &co};
    const CUresult r = g.launch(g.grid, blocks(chunkSize), 1, 1, 32, 1, 1, 0, CUstream(stream), args, nullptr);
    return r ? fail("fastWindingNumberFromGridKernel launch", r) : 0;
}

int mrc_from_vector(const void* queries, const void* dipoles, const void* nodes, const void* points, const void* faces,
                    float* out, float beta, int skipFace, uint64_t n, void* stream) {
    if (!g.module) return -1;
    if (n == 0) return 0;
    size_t sz = n;
    void* args[] = {&queries, &dipoles, &nodes, &points, &faces, &out, &beta, &skipFace, &sz};
    const CUresult r = g.launch(g.vec, blocks(n), 1, 1, 32, 1, 1, 0, CUstream(stream), args, nullptr);
    return r ? fail("fastWindingNumberFromVectorKernel launch", r) : 0;
}

int mrc_from_mesh(const void* dipoles, const void* nodes, const void* points, const void* faces, float* out, float beta,
                  uint64_t chunkSize, uint64_t chunkOffset, void* stream) {
    if (!g.module) return -1;
    if (chunkSize == 0) return 0;
    size_t cs = chunkSize, co = chunkOffset;
    void* args[] = {&dipoles, &nodes, &points, &faces, &out, &beta, &cs, &co};
    const CUresult r = g.launch(g.mesh, blocks(chunkSize), 1, 1, 32, 1, 1, 0, CUstream(stream), args, nullptr);
    return r ? fail("fastWindingNumberFromMeshKernel launch", r) : 0;
}

// Loads the projection kernel (after mrc_load, which sets up the driver and the context).
int mrc_load_projector(const char* cubin, const char* ptx) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g.projModule) return 0;
    if (!g.module) {
        std::snprintf(g_err, sizeof(g_err), "mrc_load must succeed first");
        return -1;
    }
    CUmodule m = nullptr;
    CUresult r = cubin && *cubin ? g.moduleLoad(&m, cubin) : CUDA_ERROR_FILE_NOT_FOUND;
    if (r && ptx && *ptx) r = g.moduleLoad(&m, ptx);
    if (r) return fail("cuModuleLoad (reference projector)", r);
    if ((r = g.getFunction(&g.proj, m, kProj))) return fail("projector kernel", r);
    g.projModule = m;
    return 0;
}

// The reference's projection kernel: xf maps the points, refXf the tree (NULL = identity), as its host
// class passes them after folding a rigid refXf into xf (MRCudaPointsToMeshProjector.cpp:75-102).
// out: n records of 32 bytes (MeshProjectionResult).
int mrc_project(const void* queries, const void* nodes, const void* points, const void* faces, void* out, const float* xf,
                const float* refXf, float upDistLimitSq, float loDistLimitSq, uint64_t n, void* stream) {
    if (!g.proj) return -1;
    if (n == 0) return 0;
    Matrix4 a = matrix(xf), b = matrix(refXf);
    size_t sz = n;
    void* args[] = {&queries, &nodes, &points, &faces, &out, &a, &b, &upDistLimitSq, &loDistLimitSq, &sz};
    const CUresult r = g.launch(g.proj, unsigned((n + 639) / 640), 1, 1, 640, 1, 1, 0, CUstream(stream), args, nullptr);
    return r ? fail("projector kernel launch", r) : 0;
}

}  // extern "C"
