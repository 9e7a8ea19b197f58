// C ABI (include/gbfwn.h): handle management, host <-> device staging, slab pipelining.
//
// Host-facing calls behave like MR::Cuda::FastWindingNumber (MRCuda/MRCudaFastWindingNumber.cpp):
// synchronous, results in host memory, progress reported at phase boundaries and per z-slab,
// cancellation honoured between slabs.  Without a progress callback a grid is one launch followed
// by one device->host copy; with one (or by parts) it is produced in z-slabs on one stream while
// finished slabs are copied to the host on a second stream, so the copy of slab k overlaps the
// computation of slabs k+1...
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#if defined(__linux__)
#include <sys/mman.h>
#include <unistd.h>
#endif

#include "../../include/gbfwn.h"
#include "common.cuh"
#include "handle.cuh"

using namespace gbfwn;

namespace gbfwn {
}

namespace gbfwn {

thread_local std::string g_lastError;
thread_local int g_failAllocs = 0;

int fail(int status, const std::string& msg) {
    g_lastError = msg;
    return status;
}

int cudaFail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) return fail(GBFWN_OUT_OF_MEMORY, std::string("NVIDIA GPU error: out of memory in ") + what);
    return fail(GBFWN_CUDA_ERROR, std::string("NVIDIA GPU error: ") + cudaGetErrorString(e) + " in " + what);
}

cudaError_t devMalloc(void** p, size_t bytes) {
    if (g_failAllocs > 0) {
        --g_failAllocs;
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes ? bytes : 16);
}

static constexpr int kMaxPoolDevices = 64;
static std::mutex g_poolMu;
struct PoolSlot {
    cudaMemPool_t pool = nullptr;
    bool failed = false;  // creation failed once: this device allocates with cudaMalloc from then on
};
static PoolSlot g_pools[kMaxPoolDevices];

// The pool of `device` if it exists (never creates one); null for devices without a pool.
static cudaMemPool_t existingPool(int device) {
    if (device < 0 || device >= kMaxPoolDevices) return nullptr;
    std::lock_guard<std::mutex> lk(g_poolMu);
    return g_pools[device].pool;
}

// The library's own stream-ordered pool on `device`: freed blocks stay reserved for the next
// allocation, so a handle created per call (the reference's usage) does not map its grid-sized
// staging buffer afresh every time.  gbfwn_release_cached_memory returns the reserve.  A device
// gets its pool on first use or never, so every block of a device comes from one allocator and
// poolFree can tell which one from the device alone.
cudaMemPool_t devicePool(int device) {
    if (device < 0 || device >= kMaxPoolDevices) return nullptr;
    std::lock_guard<std::mutex> lk(g_poolMu);
    PoolSlot& slot = g_pools[device];
    if (!slot.pool && !slot.failed) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
            cudaGetLastError();
            slot.failed = true;
            return nullptr;
        }
        uint64_t keep = ~uint64_t(0);
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        slot.pool = pool;
    }
    return slot.pool;
}

cudaError_t poolMalloc(void** p, size_t bytes, int device, cudaStream_t s) {
    if (g_failAllocs > 0) {
        --g_failAllocs;
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    cudaMemPool_t pool = devicePool(device);
    if (!pool) return cudaMalloc(p, bytes ? bytes : 16);
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, s);
    if (!e) e = cudaStreamSynchronize(s);  // usable from any stream once this returns
    return e;
}

void poolFree(void* p, cudaStream_t s) {
    if (!p) return;
    // the device the block lives on (not the caller's current device) decides the allocator
    int device = -1;
    cudaPointerAttributes a = {};
    if (cudaPointerGetAttributes(&a, p) == cudaSuccess) {
        device = a.device;
    } else {
        cudaGetLastError();
        cudaGetDevice(&device);
    }
    if (existingPool(device))
        cudaFreeAsync(p, s);
    else
        cudaFree(p);  // poolMalloc fell back to cudaMalloc: no pool on this device
}

}  // namespace gbfwn

namespace {
bool progress(gbfwn_progress_cb cb, void* user, float p) { return !cb || cb(p, user) != 0; }

// makeSignedByWindingNumber's update (MRVoxels/MRVDBConversions.cpp:516-530): a voxel whose winding
// number exceeds the threshold has its value negated
__global__ void flipByWindingKernel(float* __restrict__ values, const float* __restrict__ wn, int64_t n, float threshold) {
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        if (wn[i] > threshold) values[i] = -values[i];
}
}  // namespace

namespace {

bool toXf(const float* xf, Xf& out) {
    if (!xf) return false;
    for (int i = 0; i < 9; ++i) out.a[i] = xf[i];
    for (int i = 0; i < 3; ++i) out.b[i] = xf[9 + i];
    return true;
}

DistOpts toOpts(const gbfwn_dist_opts* o) {
    DistOpts d;
    if (!o) {
        d = DistOpts{0.f, FLT_MAX, 1, 0.5f, 2.f};
    } else {
        d = DistOpts{o->minDistSq, o->maxDistSq, o->nullOutsideMinMax, o->windingNumberThreshold, o->windingNumberBeta};
    }
    return d;
}

bool validDims(const int32_t* dims) {
    return dims && dims[0] > 0 && dims[1] > 0 && dims[2] > 0 && gridTiles(dims[0], dims[1], dims[2]) <= kMaxTilesPerLaunch;
}

int createCommon(gbfwn_mesh_s* h, const std::string& where) {
    std::string err;
    ListAllocator tmp;  // build work arrays, freed once the build has finished
    tmp.device = h->device;
    tmp.stream = h->stream;
    cudaError_t e = buildDeviceTree(h->dVerts, h->nv, h->dTris, h->nt, h->tree, h->treeMem, tmp, h->stream, err);
    cudaStreamSynchronize(h->stream);
    tmp.freeAll();
    h->applySignReuse();
    if (e == cudaErrorInvalidValue && !err.empty()) return fail(GBFWN_INVALID, err);
    if (e) return cudaFail(e, where.c_str());
    return GBFWN_OK;
}

int newHandle(int device, gbfwn_mesh_s** out) {
    auto* h = new gbfwn_mesh_s;
    h->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (!e) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (!e) e = cudaStreamCreateWithFlags(&h->copyStream, cudaStreamNonBlocking);
    h->treeMem.device = device;
    h->treeMem.stream = h->stream;
    if (!e) e = h->treeMem.alloc((void**)&h->scratch, 64);
    if (!e) e = cudaMemsetAsync(h->scratch, 0, 64, h->stream);
    if (e) {
        int st = cudaFail(e, "gbfwn_create");
        gbfwn_destroy(h);
        return st;
    }
    *out = h;
    return GBFWN_OK;
}

// The handle's grid work buffer (column hand-over words, inside bits and crossing lists of a grid
// launch on stream s), at least `need` bytes, grown on the handle's stream (a launch on another
// stream waits for the growth); nullptr when it cannot grow, and the launch runs without it.
void* workFor(gbfwn_mesh_s* h, size_t need, cudaStream_t s, size_t* bytes) {
    *bytes = 0;
    if (need == 0) return nullptr;
    if (h->colCap < need) {
        if (h->ensure(&h->colBuf, &h->colCap, need)) {
            cudaGetLastError();
            return nullptr;
        }
        if (s != h->stream) cudaStreamSynchronize(h->stream);
    }
    *bytes = h->colCap;
    return h->colBuf;
}

float* colStateFor(gbfwn_mesh_s* h, const GridRange& r, const Xf& X, const DistOpts& o, cudaStream_t s, size_t* bytes) {
    return static_cast<float*>(workFor(h, gridSdfColumnStateBytes(h->tree.q, r, X, o), s, bytes));
}

int refitCommon(gbfwn_mesh_s* h, const uint64_t* dChanged, cudaStream_t s, const char* what) {
    ListAllocator tmp;  // refit work arrays
    tmp.device = h->device;
    tmp.stream = s;
    cudaError_t e = refitDeviceTree(h->dVerts, h->nv, h->dTris, dChanged, h->tree, h->treeMem, tmp, s);
    cudaStreamSynchronize(s);
    tmp.freeAll();
    h->applySignReuse();
    return e ? cudaFail(e, what) : GBFWN_OK;
}

}  // namespace

extern "C" {

GBFWN_API const char* gbfwn_version(void) { return "gbfwn 0.1 (sm_103a)"; }

GBFWN_API const char* gbfwn_last_error(void) { return g_lastError.c_str(); }

GBFWN_API void gbfwn_debug_fail_next_allocs(int count) { g_failAllocs = count; }

GBFWN_API int gbfwn_release_cached_memory(int device) {
    DeviceGuard g(device);
    cudaMemPool_t pool = existingPool(device);
    if (pool) {
        cudaDeviceSynchronize();
        cudaMemPoolTrimTo(pool, 0);
    }
    return gbfwn_mc_release_workspace(device);
}

GBFWN_API void gbfwn_set_precise(gbfwn_handle h, int precise) {
    if (h) h->precise = precise ? 1 : 0;
}

GBFWN_API void gbfwn_set_sign_reuse(gbfwn_handle h, int enable) {
    if (!h) return;
    std::lock_guard<std::mutex> lk(h->mu);
    h->signReuse = enable ? 1 : 0;
    h->applySignReuse();
}

GBFWN_API int gbfwn_is_closed(gbfwn_handle h) { return h && h->tree.closed ? 1 : 0; }

GBFWN_API int gbfwn_create(const float* verts, int64_t nv, const int32_t* tris, int64_t nt, int device, gbfwn_handle* out) {
    if (!out || nv < 0 || nt < 0 || (nv > 0 && !verts) || (nt > 0 && !tris)) return fail(GBFWN_INVALID, "gbfwn_create: bad arguments");
    if (nt > INT32_MAX / 2) return fail(GBFWN_INVALID, "gbfwn_create: too many triangles");
    *out = nullptr;
    gbfwn_mesh_s* h = nullptr;
    int st = newHandle(device, &h);
    if (st) {
        // no device: an out-of-range vertex id is still reported as such (on a device the tree
        // build's face validation rejects it before any vertex is read)
        int32_t maxId = -1;
        for (int64_t i = 0; i < 3 * nt; ++i) maxId = tris[i] > maxId ? tris[i] : maxId;
        if (maxId >= nv) return fail(GBFWN_INVALID, "gbfwn_create: triangle vertex id out of range");
        return st;
    }
    DeviceGuard g(device);
    h->nv = nv;
    h->nt = nt;
    cudaError_t e = h->treeMem.alloc((void**)&h->dVerts, sizeof(float) * 3 * size_t(nv));
    if (!e) e = h->treeMem.alloc((void**)&h->dTris, sizeof(int32_t) * 3 * size_t(nt));
    if (!e && nv) e = cudaMemcpyAsync(h->dVerts, verts, sizeof(float) * 3 * size_t(nv), cudaMemcpyHostToDevice, h->stream);
    if (!e && nt) e = cudaMemcpyAsync(h->dTris, tris, sizeof(int32_t) * 3 * size_t(nt), cudaMemcpyHostToDevice, h->stream);
    if (e) {
        st = cudaFail(e, "gbfwn_create upload");
        gbfwn_destroy(h);
        return st;
    }
    if ((st = createCommon(h, "gbfwn_create"))) {
        gbfwn_destroy(h);
        return st;
    }
    *out = h;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_create_dev(const float* d_verts, int64_t nv, const int32_t* d_tris, int64_t nt, int device,
                               gbfwn_handle* out) {
    if (!out || nv < 0 || nt < 0 || (nv > 0 && !d_verts) || (nt > 0 && !d_tris)) return fail(GBFWN_INVALID, "gbfwn_create_dev: bad arguments");
    if (nt > INT32_MAX / 2) return fail(GBFWN_INVALID, "gbfwn_create_dev: too many triangles");
    *out = nullptr;
    gbfwn_mesh_s* h = nullptr;
    int st = newHandle(device, &h);
    if (st) return st;
    DeviceGuard g(device);
    h->nv = nv;
    h->nt = nt;
    cudaError_t e = h->treeMem.alloc((void**)&h->dVerts, sizeof(float) * 3 * size_t(nv));
    if (!e) e = h->treeMem.alloc((void**)&h->dTris, sizeof(int32_t) * 3 * size_t(nt));
    if (!e && nv) e = cudaMemcpyAsync(h->dVerts, d_verts, sizeof(float) * 3 * size_t(nv), cudaMemcpyDeviceToDevice, h->stream);
    if (!e && nt) e = cudaMemcpyAsync(h->dTris, d_tris, sizeof(int32_t) * 3 * size_t(nt), cudaMemcpyDeviceToDevice, h->stream);
    if (e) {
        st = cudaFail(e, "gbfwn_create_dev copy");
        gbfwn_destroy(h);
        return st;
    }
    if ((st = createCommon(h, "gbfwn_create_dev"))) {
        gbfwn_destroy(h);
        return st;
    }
    *out = h;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_destroy(gbfwn_handle h) {
    if (!h) return GBFWN_OK;
    if (h->batchRefs.load() > 0)
        return fail(GBFWN_INVALID, "gbfwn_destroy: the mesh is part of a live batch; destroy the batch first");
    {
        DeviceGuard g(h->device);
        // everything goes back to the device's pool; the device is idle first (as cudaFree would
        // make it), since a _dev call may have used the handle's arrays on a caller's stream
        cudaDeviceSynchronize();
        h->treeMem.freeAll();
        poolFree(h->outBuf, h->stream);
        poolFree(h->inBuf, h->stream);
        poolFree(h->sortBuf, h->stream);
        poolFree(h->colBuf, h->stream);
        if (h->stream) cudaStreamSynchronize(h->stream);
        for (auto ev : h->events) cudaEventDestroy(ev);
        if (h->stream) cudaStreamDestroy(h->stream);
        if (h->copyStream) cudaStreamDestroy(h->copyStream);
    }
    delete h;
    return GBFWN_OK;
}

GBFWN_API int gbfwn_refit(gbfwn_handle h, const float* verts, const uint64_t* changedVerts) {
    if (!h || (h->nv > 0 && !verts)) return fail(GBFWN_INVALID, "gbfwn_refit: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    cudaError_t e = h->nv ? cudaMemcpyAsync(h->dVerts, verts, sizeof(float) * 3 * size_t(h->nv), cudaMemcpyHostToDevice, h->stream)
                          : cudaSuccess;
    uint64_t* dBits = nullptr;
    const size_t words = size_t((h->nv + 63) / 64);
    if (!e && changedVerts && words) {
        e = devMalloc((void**)&dBits, words * sizeof(uint64_t));
        if (!e) e = cudaMemcpyAsync(dBits, changedVerts, words * sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream);
    }
    const int st = e ? cudaFail(e, "gbfwn_refit") : refitCommon(h, changedVerts ? dBits : nullptr, h->stream, "gbfwn_refit");
    if (dBits) cudaFree(dBits);
    return st;
}

GBFWN_API int gbfwn_refit_dev(gbfwn_handle h, const float* d_verts, const uint64_t* d_changedVerts, void* stream) {
    if (!h || (h->nv > 0 && !d_verts)) return fail(GBFWN_INVALID, "gbfwn_refit_dev: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    const cudaError_t e = (h->nv && d_verts != h->dVerts)
                              ? cudaMemcpyAsync(h->dVerts, d_verts, sizeof(float) * 3 * size_t(h->nv), cudaMemcpyDeviceToDevice, s)
                              : cudaSuccess;
    return e ? cudaFail(e, "gbfwn_refit_dev") : refitCommon(h, d_changedVerts, s, "gbfwn_refit_dev");
}

GBFWN_API int64_t gbfwn_num_faces(gbfwn_handle h) { return h ? h->nt : 0; }
GBFWN_API int64_t gbfwn_num_nodes(gbfwn_handle h) { return h && h->tree.nLeaves ? 2 * h->tree.nLeaves - 1 : 0; }

GBFWN_API int gbfwn_get_tree(gbfwn_handle h, void* nodes, float* dipoles) {
    if (!h) return fail(GBFWN_INVALID, "gbfwn_get_tree: null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    const int64_t n = gbfwn_num_nodes(h);
    if (n == 0) return GBFWN_OK;
    cudaError_t e = cudaSuccess;
    if (nodes) e = cudaMemcpyAsync(nodes, h->tree.nodes, sizeof(RefNode) * size_t(n), cudaMemcpyDeviceToHost, h->stream);
    if (!e && dipoles) e = cudaMemcpyAsync(dipoles, h->tree.dip8, sizeof(float) * 8 * size_t(n), cudaMemcpyDeviceToHost, h->stream);
    if (!e) e = cudaStreamSynchronize(h->stream);
    if (e) return cudaFail(e, "gbfwn_get_tree");
    return GBFWN_OK;
}

// ------------------------------------------------------------------------- device-pointer calls
namespace {
// Spatially coherent processing order for n >= 8192 arbitrary points (Morton order inside the mesh
// box); null for small inputs, which are processed as given.
cudaError_t pointOrder(gbfwn_mesh_s* h, const float* d_pts, int64_t n, cudaStream_t s, const int32_t** order) {
    *order = nullptr;
    if (n < 8192 || h->tree.nLeaves == 0) return cudaSuccess;
    const size_t words = size_t(n) + size_t(mortonOrderScratch(n));
    cudaError_t e = h->ensure(&h->sortBuf, &h->sortCap, words * sizeof(int32_t));
    if (e) return e;
    int32_t* buf = static_cast<int32_t*>(h->sortBuf);
    const float lo[3] = {h->tree.q.rootBox0.x, h->tree.q.rootBox0.y, h->tree.q.rootBox0.z};
    const float hi[3] = {h->tree.q.rootBox1.x, h->tree.q.rootBox1.y, h->tree.q.rootBox1.z};
    e = mortonOrder(d_pts, n, lo, hi, buf, buf + n, s);
    if (!e) *order = buf;
    return e;
}
}  // namespace

GBFWN_API int gbfwn_from_vector_dev(gbfwn_handle h, const float* d_pts, int64_t n, float beta, int32_t skipFace,
                                    float* d_out, void* stream) {
    if (!h || n < 0 || (n > 0 && (!d_pts || !d_out))) return fail(GBFWN_INVALID, "gbfwn_from_vector_dev: bad arguments");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    const int32_t* order = nullptr;
    cudaError_t e = pointOrder(h, d_pts, n, s, &order);
    if (!e) e = launchVectorFwn(h->tree.q, d_pts, n, beta, skipFace, h->precise, d_out, h->scratch, s, order);
    return e ? cudaFail(e, "gbfwn_from_vector_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_vector_with_distances_dev(gbfwn_handle h, const float* d_pts, int64_t n, const gbfwn_dist_opts* opts,
                                              float* d_out, void* stream) {
    if (!h || n < 0 || (n > 0 && (!d_pts || !d_out))) return fail(GBFWN_INVALID, "gbfwn_vector_with_distances_dev: bad arguments");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    const int32_t* order = nullptr;
    cudaError_t e = pointOrder(h, d_pts, n, s, &order);
    if (!e) e = launchVectorSdf(h->tree.q, d_pts, n, toOpts(opts), h->precise, d_out, h->scratch, s, order);
    return e ? cudaFail(e, "gbfwn_vector_with_distances_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_self_intersections_dev(gbfwn_handle h, float beta, uint64_t* d_bits, float* d_wn, void* stream) {
    if (!h || !d_bits) return fail(GBFWN_INVALID, "gbfwn_self_intersections_dev: bad arguments");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    cudaError_t e = launchSelfIntersections(h->tree.q, beta, h->precise, d_bits, d_wn, h->scratch, s);
    return e ? cudaFail(e, "gbfwn_self_intersections_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_from_grid_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12], float beta, float* d_out,
                                  void* stream) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !d_out) return fail(GBFWN_INVALID, "gbfwn_from_grid_dev: bad arguments");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    GridRange r{dims[0], dims[1], dims[2], 0, dims[2], 0};
    cudaError_t e = launchGridFwn(h->tree.q, r, X, beta, h->precise, d_out, h->scratch, s);
    return e ? cudaFail(e, "gbfwn_from_grid_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_make_signed_by_winding_number_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                      float beta, float threshold, float* d_values, void* stream) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !d_values)
        return fail(GBFWN_INVALID, "gbfwn_make_signed_by_winding_number_dev: bad arguments");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    const int64_t n = int64_t(dims[0]) * dims[1] * dims[2];
    if (signColumnsApply(h->tree.q, X, beta, threshold)) {  // closed mesh, z axis vertical: one ray per column
        GridRange r{dims[0], dims[1], dims[2], 0, dims[2], 0};
        size_t workBytes = 0;
        void* work = workFor(h, signColumnsWorkBytes(r), s, &workBytes);
        const cudaError_t e =
            launchSignColumns(h->tree.q, r, X, beta, threshold, h->precise, nullptr, d_values, work, workBytes, h->scratch, s);
        return e ? cudaFail(e, "gbfwn_make_signed_by_winding_number_dev") : GBFWN_OK;
    }
    float* wn = nullptr;
    cudaError_t e = g_failAllocs > 0 ? (--g_failAllocs, cudaErrorMemoryAllocation)
                                     : cudaMallocAsync((void**)&wn, sizeof(float) * size_t(n), s);
    if (e) return cudaFail(e, "gbfwn_make_signed_by_winding_number_dev");
    GridRange r{dims[0], dims[1], dims[2], 0, dims[2], 0};
    e = launchGridFwn(h->tree.q, r, X, beta, h->precise, wn, h->scratch, s);
    if (!e) {
        flipByWindingKernel<<<unsigned(std::min<int64_t>((n + 255) / 256, int64_t(numSMs()) * 16)), 256, 0, s>>>(d_values, wn, n,
                                                                                                           threshold);
        e = cudaGetLastError();
    }
    const cudaError_t ef = cudaFreeAsync(wn, s);
    if (!e) e = ef;
    return e ? cudaFail(e, "gbfwn_make_signed_by_winding_number_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_from_grid_with_distances_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                 const gbfwn_dist_opts* opts, float* d_out, void* stream) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !d_out) return fail(GBFWN_INVALID, "gbfwn_from_grid_with_distances_dev: bad arguments");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    GridRange r{dims[0], dims[1], dims[2], 0, dims[2], 0};
    const DistOpts o = toOpts(opts);
    size_t colBytes = 0;
    float* col = colStateFor(h, r, X, o, s, &colBytes);
    cudaError_t e = launchGridSdf(h->tree.q, r, X, o, h->precise, d_out, h->scratch, s, col, colBytes);
    return e ? cudaFail(e, "gbfwn_from_grid_with_distances_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_from_grid_slab_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12], float beta, int32_t z0,
                                       int32_t z1, float* d_out, void* stream) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !d_out || z0 < 0 || z1 > dims[2] || z0 >= z1)
        return fail(GBFWN_INVALID, "gbfwn_from_grid_slab_dev: bad arguments");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    GridRange r{dims[0], dims[1], dims[2], z0, z1, z0};
    cudaError_t e = launchGridFwn(h->tree.q, r, X, beta, h->precise, d_out, h->scratch, s);
    return e ? cudaFail(e, "gbfwn_from_grid_slab_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_from_grid_with_distances_slab_dev(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                      const gbfwn_dist_opts* opts, int32_t z0, int32_t z1, float* d_out,
                                                      void* stream) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !d_out || z0 < 0 || z1 > dims[2] || z0 >= z1)
        return fail(GBFWN_INVALID, "gbfwn_from_grid_with_distances_slab_dev: bad arguments");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    GridRange r{dims[0], dims[1], dims[2], z0, z1, z0};
    const DistOpts o = toOpts(opts);
    size_t colBytes = 0;
    float* col = colStateFor(h, r, X, o, s, &colBytes);
    cudaError_t e = launchGridSdf(h->tree.q, r, X, o, h->precise, d_out, h->scratch, s, col, colBytes);
    return e ? cudaFail(e, "gbfwn_from_grid_with_distances_slab_dev") : GBFWN_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------- host-memory calls
namespace {

// True when the kernel can write the `bytes` at host address p itself: the device accesses pageable
// host memory through the CPU's page tables (cudaDevAttrPageableMemoryAccess: Grace-Blackwell's
// coherent NVLink-C2C) and every page of the range is already populated (mincore), as a
// std::vector that was resized or a buffer reused from an earlier call is.  A GPU write to a page the
// CPU has not touched yet takes a page fault (measured on GB300: about 0.35 ms per MB, far slower
// than a copy), so such ranges, and every other platform, take the device buffer + copy path.
bool directHostWritable(int device, const void* p, size_t bytes) {
#if defined(__linux__)
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (!pageable || !p || bytes == 0) return false;
    const long page = sysconf(_SC_PAGESIZE);
    if (page <= 0) return false;
    const uintptr_t a = reinterpret_cast<uintptr_t>(p), lo = a & ~uintptr_t(page - 1), hi = a + bytes;
    std::vector<unsigned char> resident((hi - lo + size_t(page) - 1) / size_t(page));
    if (mincore(reinterpret_cast<void*>(lo), hi - lo, resident.data()) != 0) return false;
    for (unsigned char v : resident)
        if (!(v & 1)) return false;
    return true;
#else
    (void)device;
    (void)p;
    (void)bytes;
    return false;
#endif
}

// Computes a grid in slabs of whole XY layers.  Each slab's kernel writes into the device output
// buffer; the copy stream waits for it and moves it to `hostOut` (if not null) and/or hands it to
// `slab` (by-parts mode, with `overlap` layers shared between consecutive slabs).
template <typename LaunchFn>
int runGrid(gbfwn_mesh_s* h, const int32_t dims[3], LaunchFn launch, float* hostOut, int32_t overlap, int32_t maxLayers,
            gbfwn_slab_cb slab, void* slabUser, gbfwn_progress_cb cb, void* user, const char* what) {
    const size_t layer = size_t(dims[0]) * dims[1];
    const int nz = dims[2];
    if (!progress(cb, user, 0.f)) return fail(GBFWN_CANCELLED, "operation canceled");
    // slab height: about 16 M voxels per slab in by-parts mode (the callback's memory), 64 M with a
    // progress callback (progress / cancellation granularity), at least 1 layer; without either the
    // whole grid is one launch (the device->host copy runs at C2C speed, ~3 ms for 537 MB on GB300,
    // while splitting the launch costs more: every launch drains its persistent grid and restarts the
    // seeded column walk)
    int slabLayers = int(std::max<size_t>(1, (size_t(16) << 20) / layer));
    if (!slab) slabLayers = cb ? int(std::max<size_t>(1, (size_t(64) << 20) / layer)) : nz;
    if (maxLayers > 0) slabLayers = std::min(slabLayers, int(maxLayers));
    if (overlap < 0) overlap = 0;
    if (slab && slabLayers <= overlap) slabLayers = overlap + 1;
    slabLayers = std::min(slabLayers, nz);
    struct SlabR {
        int z0, z1;  // layers computed [z0, z1)
    };
    std::vector<SlabR> slabs;
    if (!slab) {
        for (int z = 0; z < nz; z += slabLayers) slabs.push_back({z, std::min(nz, z + slabLayers)});
    } else {
        // MRMesh/MRChunkIterator.h:44-47 semantics: chunks of slabLayers layers stepping by
        // slabLayers - overlap
        const int step = slabLayers - overlap;
        for (int z = 0;; z += step) {
            const int z1 = std::min(nz, z + slabLayers);
            slabs.push_back({z, z1});
            if (z1 >= nz) break;
        }
    }
    // device buffer: the whole grid in host mode, two slab buffers in by-parts mode
    const bool whole = !slab;
    cudaError_t e = cudaSuccess;
    // one launch straight into the caller's memory when the GPU can write it in place (no device
    // buffer, no copy: the results cross NVLink-C2C as the kernel stores them)
    if (whole && hostOut && !cb && slabs.size() == 1 && directHostWritable(h->device, hostOut, layer * size_t(nz) * sizeof(float))) {
        if ((e = h->resetStatus(h->stream))) return cudaFail(e, what);
        GridRange r{dims[0], dims[1], dims[2], 0, nz, 0};
        if ((e = launch(r, hostOut, h->stream))) return cudaFail(e, what);
        if ((e = cudaStreamSynchronize(h->stream))) return cudaFail(e, what);
        return h->checkStatus();
    }
    const size_t slabBytes = layer * size_t(slabLayers) * sizeof(float);
    const size_t need = whole ? layer * size_t(nz) * sizeof(float) : 2 * slabBytes;
    e = h->ensure(&h->outBuf, &h->outCap, need);
    if (!e) e = h->ensureEvents(2 * slabs.size() + 2);
    if (e) return cudaFail(e, what);
    if ((e = h->resetStatus(h->stream))) return cudaFail(e, what);
    float* dOut = (float*)h->outBuf;
    std::vector<float> pinnedless;  // by-parts host slab
    if (slab) pinnedless.resize(layer * size_t(slabLayers));
    // in by-parts mode slab i reuses buffer i%2, so the kernel of slab i waits for the copy of slab i-2
    for (size_t i = 0; i < slabs.size(); ++i) {
        const SlabR& sr = slabs[i];
        float* buf = whole ? dOut + layer * size_t(sr.z0) : dOut + (i % 2) * (slabBytes / sizeof(float));
        if (!whole && i >= 2) cudaStreamWaitEvent(h->stream, h->events[2 * (i - 2) + 1], 0);
        GridRange r{dims[0], dims[1], dims[2], sr.z0, sr.z1, sr.z0};
        if ((e = launch(r, buf, h->stream))) return cudaFail(e, what);
        cudaEventRecord(h->events[2 * i], h->stream);
        if (!whole) {
            // by-parts: launches run ahead by at most one slab; hand slabs over in order
            if (i >= 1) {
                const size_t j = i - 1;
                const SlabR& pr = slabs[j];
                const float* pbuf = dOut + (j % 2) * (slabBytes / sizeof(float));
                const size_t cnt = layer * size_t(pr.z1 - pr.z0);
                cudaStreamWaitEvent(h->copyStream, h->events[2 * j], 0);
                if ((e = cudaMemcpyAsync(pinnedless.data(), pbuf, cnt * sizeof(float), cudaMemcpyDeviceToHost, h->copyStream)))
                    return cudaFail(e, what);
                cudaEventRecord(h->events[2 * j + 1], h->copyStream);
                if ((e = cudaStreamSynchronize(h->copyStream))) return cudaFail(e, what);
                const int32_t sd[3] = {dims[0], dims[1], pr.z1 - pr.z0};
                const int rc = slab(pinnedless.data(), sd, pr.z0, slabUser);
                if (rc) {
                    cudaStreamSynchronize(h->stream);
                    return fail(rc, "slab callback returned an error");
                }
                if (!progress(cb, user, float(j + 1) / float(slabs.size()))) {
                    cudaStreamSynchronize(h->stream);
                    return fail(GBFWN_CANCELLED, "operation canceled");
                }
            }
        }
    }
    if (whole) {
        for (size_t i = 0; i < slabs.size(); ++i) {
            const SlabR& sr = slabs[i];
            const size_t off = layer * size_t(sr.z0), cnt = layer * size_t(sr.z1 - sr.z0);
            cudaStreamWaitEvent(h->copyStream, h->events[2 * i], 0);
            if (hostOut && (e = cudaMemcpyAsync(hostOut + off, dOut + off, cnt * sizeof(float), cudaMemcpyDeviceToHost, h->copyStream)))
                return cudaFail(e, what);
            if (cb) {
                if ((e = cudaStreamSynchronize(h->copyStream))) return cudaFail(e, what);
                if (!progress(cb, user, float(i + 1) / float(slabs.size()))) {
                    cudaStreamSynchronize(h->stream);
                    return fail(GBFWN_CANCELLED, "operation canceled");
                }
            }
        }
        if ((e = cudaStreamSynchronize(h->copyStream))) return cudaFail(e, what);
    } else {
        const size_t j = slabs.size() - 1;
        const SlabR& pr = slabs[j];
        const float* pbuf = dOut + (j % 2) * (slabBytes / sizeof(float));
        const size_t cnt = layer * size_t(pr.z1 - pr.z0);
        cudaStreamWaitEvent(h->copyStream, h->events[2 * j], 0);
        if ((e = cudaMemcpyAsync(pinnedless.data(), pbuf, cnt * sizeof(float), cudaMemcpyDeviceToHost, h->copyStream)))
            return cudaFail(e, what);
        if ((e = cudaStreamSynchronize(h->copyStream))) return cudaFail(e, what);
        int stc = h->checkStatus();
        if (stc) return stc;
        const int32_t sd[3] = {dims[0], dims[1], pr.z1 - pr.z0};
        const int rc = slab(pinnedless.data(), sd, pr.z0, slabUser);
        if (rc) return fail(rc, "slab callback returned an error");
        if (!progress(cb, user, 1.f)) return fail(GBFWN_CANCELLED, "operation canceled");
    }
    if ((e = cudaStreamSynchronize(h->stream))) return cudaFail(e, what);
    return h->checkStatus();
}

template <typename LaunchFn>
int runPoints(gbfwn_mesh_s* h, const float* pts, int64_t n, float* out, LaunchFn launch, gbfwn_progress_cb cb, void* user,
              const char* what) {
    if (!progress(cb, user, 0.f)) return fail(GBFWN_CANCELLED, "operation canceled");
    if (n == 0) return progress(cb, user, 1.f) ? GBFWN_OK : fail(GBFWN_CANCELLED, "operation canceled");
    cudaError_t e = h->ensure(&h->inBuf, &h->inCap, sizeof(float) * 3 * size_t(n));
    if (!e) e = h->ensure(&h->outBuf, &h->outCap, sizeof(float) * size_t(n));
    if (!e) e = h->resetStatus(h->stream);
    if (!e) e = cudaMemcpyAsync(h->inBuf, pts, sizeof(float) * 3 * size_t(n), cudaMemcpyHostToDevice, h->stream);
    if (e) return cudaFail(e, what);
    if ((e = launch((const float*)h->inBuf, (float*)h->outBuf, h->stream))) return cudaFail(e, what);
    if ((e = cudaMemcpyAsync(out, h->outBuf, sizeof(float) * size_t(n), cudaMemcpyDeviceToHost, h->stream))) return cudaFail(e, what);
    if ((e = cudaStreamSynchronize(h->stream))) return cudaFail(e, what);
    int st = h->checkStatus();
    if (st) return st;
    return progress(cb, user, 1.f) ? GBFWN_OK : fail(GBFWN_CANCELLED, "operation canceled");
}

}  // namespace

extern "C" {

GBFWN_API int gbfwn_from_vector(gbfwn_handle h, const float* pts, int64_t n, float beta, int32_t skipFace, float* out,
                                gbfwn_progress_cb cb, void* user) {
    if (!h || n < 0 || (n > 0 && (!pts || !out))) return fail(GBFWN_INVALID, "gbfwn_from_vector: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    return runPoints(
        h, pts, n, out,
        [&](const float* dp, float* dout, cudaStream_t s) {
            const int32_t* order = nullptr;
            cudaError_t oe = pointOrder(h, dp, n, s, &order);
            return oe ? oe : launchVectorFwn(h->tree.q, dp, n, beta, skipFace, h->precise, dout, h->scratch, s, order);
        },
        cb, user, "gbfwn_from_vector");
}

GBFWN_API int gbfwn_vector_with_distances(gbfwn_handle h, const float* pts, int64_t n, const gbfwn_dist_opts* opts,
                                          float* out, gbfwn_progress_cb cb, void* user) {
    if (!h || n < 0 || (n > 0 && (!pts || !out))) return fail(GBFWN_INVALID, "gbfwn_vector_with_distances: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    const DistOpts o = toOpts(opts);
    return runPoints(
        h, pts, n, out,
        [&](const float* dp, float* dout, cudaStream_t s) {
            const int32_t* order = nullptr;
            cudaError_t oe = pointOrder(h, dp, n, s, &order);
            return oe ? oe : launchVectorSdf(h->tree.q, dp, n, o, h->precise, dout, h->scratch, s, order);
        },
        cb, user, "gbfwn_vector_with_distances");
}

GBFWN_API int gbfwn_self_intersections(gbfwn_handle h, float beta, uint64_t* bits, float* wn, gbfwn_progress_cb cb,
                                       void* user) {
    if (!h || !bits) return fail(GBFWN_INVALID, "gbfwn_self_intersections: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    if (!progress(cb, user, 0.f)) return fail(GBFWN_CANCELLED, "operation canceled");
    const size_t words = size_t((h->nt + 63) / 64);
    const size_t bytes = words * sizeof(uint64_t) + (wn ? sizeof(float) * size_t(h->nt) : 0);
    cudaError_t e = h->ensure(&h->outBuf, &h->outCap, bytes + 16);
    if (!e) e = h->resetStatus(h->stream);
    if (e) return cudaFail(e, "gbfwn_self_intersections");
    uint64_t* dBits = (uint64_t*)h->outBuf;
    float* dWn = wn ? (float*)(dBits + words) : nullptr;
    if ((e = launchSelfIntersections(h->tree.q, beta, h->precise, dBits, dWn, h->scratch, h->stream)))
        return cudaFail(e, "gbfwn_self_intersections");
    if (words && (e = cudaMemcpyAsync(bits, dBits, words * sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream)))
        return cudaFail(e, "gbfwn_self_intersections");
    if (wn && h->nt && (e = cudaMemcpyAsync(wn, dWn, sizeof(float) * size_t(h->nt), cudaMemcpyDeviceToHost, h->stream)))
        return cudaFail(e, "gbfwn_self_intersections");
    if ((e = cudaStreamSynchronize(h->stream))) return cudaFail(e, "gbfwn_self_intersections");
    int st = h->checkStatus();
    if (st) return st;
    return progress(cb, user, 1.f) ? GBFWN_OK : fail(GBFWN_CANCELLED, "operation canceled");
}

GBFWN_API int gbfwn_from_grid(gbfwn_handle h, const int32_t dims[3], const float xf[12], float beta, float* out,
                              gbfwn_progress_cb cb, void* user) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !out) return fail(GBFWN_INVALID, "gbfwn_from_grid: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    return runGrid(
        h, dims,
        [&](const GridRange& r, float* buf, cudaStream_t s) {
            return launchGridFwn(h->tree.q, r, X, beta, h->precise, buf, h->scratch, s);
        },
        out, 0, 0, nullptr, nullptr, cb, user, "gbfwn_from_grid");
}

GBFWN_API int gbfwn_from_grid_with_distances(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                             const gbfwn_dist_opts* opts, float* out, gbfwn_progress_cb cb, void* user) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !out) return fail(GBFWN_INVALID, "gbfwn_from_grid_with_distances: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    const DistOpts o = toOpts(opts);
    return runGrid(
        h, dims,
        [&](const GridRange& r, float* buf, cudaStream_t s) {
            size_t colBytes = 0;
            float* col = colStateFor(h, r, X, o, s, &colBytes);
            return launchGridSdf(h->tree.q, r, X, o, h->precise, buf, h->scratch, s, col, colBytes);
        },
        out, 0, 0, nullptr, nullptr, cb, user, "gbfwn_from_grid_with_distances");
}

GBFWN_API int gbfwn_from_grid_by_parts(gbfwn_handle h, const int32_t dims[3], const float xf[12], float beta,
                                       int32_t layerOverlap, int32_t maxLayersPerSlab, gbfwn_slab_cb slab,
                                       void* slabUser, gbfwn_progress_cb cb, void* user) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !slab || layerOverlap < 0)
        return fail(GBFWN_INVALID, "gbfwn_from_grid_by_parts: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    return runGrid(
        h, dims,
        [&](const GridRange& r, float* buf, cudaStream_t s) {
            return launchGridFwn(h->tree.q, r, X, beta, h->precise, buf, h->scratch, s);
        },
        nullptr, layerOverlap, maxLayersPerSlab, slab, slabUser, cb, user, "gbfwn_from_grid_by_parts");
}

GBFWN_API int gbfwn_from_grid_with_distances_by_parts(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                      const gbfwn_dist_opts* opts, int32_t layerOverlap,
                                                      int32_t maxLayersPerSlab, gbfwn_slab_cb slab, void* slabUser,
                                                      gbfwn_progress_cb cb, void* user) {
    Xf X;
    if (!h || !validDims(dims) || !toXf(xf, X) || !slab || layerOverlap < 0)
        return fail(GBFWN_INVALID, "gbfwn_from_grid_with_distances_by_parts: bad arguments");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    const DistOpts o = toOpts(opts);
    return runGrid(
        h, dims,
        [&](const GridRange& r, float* buf, cudaStream_t s) {
            size_t colBytes = 0;
            float* col = colStateFor(h, r, X, o, s, &colBytes);
            return launchGridSdf(h->tree.q, r, X, o, h->precise, buf, h->scratch, s, col, colBytes);
        },
        nullptr, layerOverlap, maxLayersPerSlab, slab, slabUser, cb, user, "gbfwn_from_grid_with_distances_by_parts");
}

// Memory estimators (the reference's: MRViewer/MRCudaAccessor.cpp:162-194).  Callers compare them
// with the free device memory before choosing the GPU path, so they cover the peak, which is the
// tree build.  Kept per handle: vertices, triangles, face -> slot, the reference nodes and dipoles
// (32 B each per node, for export and refit), the wide query records (96 B closest-point + 64 B
// winding-number per internal node) and leaf triangles (48 B): 352 B per face.  Build work arrays,
// all alive until the build ends: two 40-byte leaf records and two 16-byte sort keys, flags, ranks and
// ranges per node, segment lists and histograms, parents, arrival counters and oriented-box
// bookkeeping: under 244 B per face.  32 MiB cover the rounding of the thirty-odd allocations.
GBFWN_API size_t gbfwn_mesh_memory(int64_t nv, int64_t nt) {
    const size_t v = size_t(std::max<int64_t>(nv, 0)), n = size_t(std::max<int64_t>(nt, 0));
    const size_t kept = v * 12 + n * (12 + 4) + (2 * n) * (32 + 32) + n * (96 + 64) + n * 48;
    const size_t build = n * 244;
    return kept + build + (size_t(32) << 20);
}
// plus the result and, for signed distances, the columns' hand-over words: 128 B per column work
// item of 16 or 32 tiles, or of fewer while under 50 items per resident warp remain
GBFWN_API size_t gbfwn_from_grid_memory(int64_t nv, int64_t nt, const int32_t dims[3]) {
    const size_t vox = dims ? size_t(std::max(dims[0], 0)) * size_t(std::max(dims[1], 0)) * size_t(std::max(dims[2], 0)) : 0;
    const size_t tiles = (dims && vox) ? size_t(gridTiles(dims[0], dims[1], dims[2])) : 0;
    const size_t items = std::min(tiles, tiles / 16 + size_t(50) * size_t(numSMs()) * 32);
    // the inside bits of a closed mesh's grid, its columns' crossing lists (72 bytes per column) and
    // the paired walk's fix list (16 bytes per two warp tiles and per work item)
    const size_t bits = dims && vox ? size_t((dims[0] + 31) / 32) * size_t(dims[1]) * size_t(dims[2]) * 4 +
                                          size_t(dims[0]) * size_t(dims[1]) * 72 + 512 + tiles * 8 + items * 16 + 32
                                    : 0;
    return gbfwn_mesh_memory(nv, nt) + vox * sizeof(float) + items * 32 * sizeof(float) + bits;
}
// staging: points in (12 B) and results out (4 B); from 8,192 points also the Morton order and its
// sort scratch (6 int32 words per point)
GBFWN_API size_t gbfwn_from_vector_memory(int64_t nv, int64_t nt, int64_t npts) {
    const size_t n = size_t(std::max<int64_t>(npts, 0));
    return gbfwn_mesh_memory(nv, nt) + n * 16 + (n >= 8192 ? n * 24 + 4096 : 0);
}
GBFWN_API size_t gbfwn_self_intersections_memory(int64_t nv, int64_t nt) {
    return gbfwn_mesh_memory(nv, nt) + size_t(std::max<int64_t>(nt, 0)) * 4 + size_t((nt + 63) / 64) * 8;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Allocation-free signed-distance grid.
//
// Some callers must not call cudaMalloc / cudaFree at the moment they need a distance grid: a host
// application that owns the whole device-memory budget and hands its plugins preallocated buffers
// only, or a latency-bound loop (an interactive viewer's frame, a tool-path planner's inner step)
// where cudaFree's implicit device-wide synchronisation or an allocation failure halfway through
// is not acceptable.  Such a caller creates the mesh handle once, at set-up time, and then calls
// gbfwn_from_grid_with_distances_noalloc with its own device output buffer.  The kernel's only
// scratch -- the work-queue ticket counter and the status word -- lives in the fixed device array
// below, which every GPU that loads this library keeps until the process exits.
namespace {

// 256 bytes per device; words [0] ticket counter, [1] status bits, the rest unused.
static __device__ __align__(256) unsigned g_noallocScratch[64];

// Device address of g_noallocScratch on the current device.  In host code the array's name is only
// a host-side stand-in, not a device address.  Looked up on every call (a host-side query that
// enqueues nothing), so a context created afresh after a device reset is seen.
int noallocScratch(unsigned** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess) return cudaFail(e, "gbfwn_from_grid_with_distances_noalloc: cudaGetSymbolAddress");
    *out = static_cast<unsigned*>(p);
    return GBFWN_OK;
}

}  // namespace

extern "C" GBFWN_API int gbfwn_from_grid_with_distances_noalloc(gbfwn_handle h, const int32_t dims[3], const float xf[12],
                                                                const gbfwn_dist_opts* opts, float* d_out, void* stream) {
    Xf X;
    if (!h || !dims || !toXf(xf, X) || !d_out || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
        return fail(GBFWN_INVALID, "gbfwn_from_grid_with_distances_noalloc: bad arguments");
    if (gridTiles(dims[0], dims[1], dims[2]) > kMaxTilesPerLaunch)
        return fail(GBFWN_INVALID,
                    "gbfwn_from_grid_with_distances_noalloc: grid too large for the fixed scratch (its 32-bit work-queue "
                    "counter covers at most 2^32-1 tiles of 4x4x2 voxels)");
    DeviceGuard g(h->device);
    unsigned* scratch = nullptr;
    if (int st = noallocScratch(&scratch)) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    // the array keeps the previous call's contents: the ticket counter and the status word must start at zero
    cudaError_t e = cudaMemsetAsync(scratch, 0, 2 * sizeof(unsigned), s);
    GridRange r{dims[0], dims[1], dims[2], 0, dims[2], 0};
    if (!e) e = launchGridSdf(h->tree.q, r, X, toOpts(opts), h->precise, d_out, scratch, s);
    return e ? cudaFail(e, "gbfwn_from_grid_with_distances_noalloc") : GBFWN_OK;
}
