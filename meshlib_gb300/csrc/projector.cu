// C ABI of the points-to-mesh projector (MR::IPointsToMeshProjector, MRMesh/MRPointsToMeshProjector.h:11-30):
// the host-side handling of the two transforms and the launch of the projection kernel (query.cu).
#include <cfloat>
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/gbfwn.h"
#include "common.cuh"
#include "handle.cuh"

using namespace gbfwn;

static_assert(sizeof(gbfwn_projection) == 32, "gbfwn_projection is the 32-byte MR::MeshProjectionResult layout");

namespace {

// Affine map in the reference's float arithmetic (MRMesh/MRAffineXf.h, MRMesh/MRMatrix3.h): rows of
// A, then b.  This file is compiled without floating-point contraction, so the products and sums
// round as the reference's do.
struct HostXf {
    float A[3][3];
    float b[3];
};

HostXf fromArray(const float* x) {
    HostXf r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.A[i][j] = x[3 * i + j];
    for (int i = 0; i < 3; ++i) r.b[i] = x[9 + i];
    return r;
}

Xf toDevice(const HostXf& x) {
    Xf r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.a[3 * i + j] = x.A[i][j];
    for (int i = 0; i < 3; ++i) r.b[i] = x.b[i];
    return r;
}

float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// MRMesh/MRMatrix3Decompose.h:27-39 isRigid: the diagonal of R in the Gram-Schmidt QR of A
// (MRMesh/MRMatrix3.h:272-294) is 1 within 10 float epsilons.
bool isRigid(const HostXf& x) {
    float a0[3], a1[3], a2[3];
    for (int i = 0; i < 3; ++i) {
        a0[i] = x.A[i][0];
        a1[i] = x.A[i][1];
        a2[i] = x.A[i][2];
    }
    const float r00 = std::sqrt(dot3(a0, a0));
    float e0[3] = {0, 0, 0}, e1[3] = {0, 0, 0};
    if (r00 > 0) {
        const float inv = 1 / r00;
        for (int i = 0; i < 3; ++i) e0[i] = a0[i] * inv;
    }
    const float r01 = dot3(e0, a1), r02 = dot3(e0, a2);
    for (int i = 0; i < 3; ++i) a1[i] -= r01 * e0[i];
    const float r11 = std::sqrt(dot3(a1, a1));
    if (r11 > 0) {
        const float inv = 1 / r11;
        for (int i = 0; i < 3; ++i) e1[i] = a1[i] * inv;
    }
    const float r12 = dot3(e1, a2);
    for (int i = 0; i < 3; ++i) a2[i] -= r02 * e0[i] + r12 * e1[i];
    const float r22 = std::sqrt(dot3(a2, a2));
    const float eps = 10 * FLT_EPSILON;
    return std::fabs(r00 - 1) <= eps && std::fabs(r11 - 1) <= eps && std::fabs(r22 - 1) <= eps;
}

// MRMesh/MRMatrix3.h:227-247 (det, cofactor inverse, zero matrix when singular) and
// MRMesh/MRAffineXf.h:51-57 (b' = -(A' b)).
HostXf inverse(const HostXf& x) {
    const auto& m = x.A;
    const float det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                      m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    HostXf r{};
    if (det != 0) {
        const float c[3][3] = {
            {m[1][1] * m[2][2] - m[1][2] * m[2][1], m[0][2] * m[2][1] - m[0][1] * m[2][2], m[0][1] * m[1][2] - m[0][2] * m[1][1]},
            {m[1][2] * m[2][0] - m[1][0] * m[2][2], m[0][0] * m[2][2] - m[0][2] * m[2][0], m[0][2] * m[1][0] - m[0][0] * m[1][2]},
            {m[1][0] * m[2][1] - m[1][1] * m[2][0], m[0][1] * m[2][0] - m[0][0] * m[2][1], m[0][0] * m[1][1] - m[0][1] * m[1][0]}};
        const float inv = 1 / det;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.A[i][j] = c[i][j] * inv;
    }
    for (int i = 0; i < 3; ++i) r.b[i] = -(r.A[i][0] * x.b[0] + r.A[i][1] * x.b[1] + r.A[i][2] * x.b[2]);
    return r;
}

// u * v: x -> u(v(x)), MRMesh/MRAffineXf.h:61-62 (A = u.A v.A row by column, b = u.A v.b + u.b)
HostXf compose(const HostXf& u, const HostXf& v) {
    HostXf r;
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) r.A[i][j] = u.A[i][0] * v.A[0][j] + u.A[i][1] * v.A[1][j] + u.A[i][2] * v.A[2][j];
        r.b[i] = (u.A[i][0] * v.b[0] + u.A[i][1] * v.b[1] + u.A[i][2] * v.b[2]) + u.b[i];
    }
    return r;
}

// MRMesh/MRMeshProject.cpp:105-121 createProjectionTransforms: a non-rigid mesh map stays on the
// mesh; otherwise the inverse of the mesh map is folded into the point map.
struct Transforms {
    bool hasPoint = false, hasTree = false;
    HostXf point{}, tree{};
};

Transforms simplify(const float* objXf, const float* refXf) {
    Transforms t;
    const bool nonRigidTree = refXf && !isRigid(fromArray(refXf));
    if (nonRigidTree) {
        t.hasTree = true;
        t.tree = fromArray(refXf);
    }
    if (nonRigidTree || !refXf) {
        if (objXf) {
            t.hasPoint = true;
            t.point = fromArray(objXf);
        }
    } else {
        t.hasPoint = true;
        t.point = inverse(fromArray(refXf));
        if (objXf) t.point = compose(t.point, fromArray(objXf));
    }
    return t;
}

// Box in the callers' point space that the mesh occupies (for the Morton order only): the root box,
// through the mesh map when there is one, back through the inverse of the point map.
bool orderBox(const gbfwn_mesh_s* h, const Transforms& tr, float lo[3], float hi[3]) {
    const float4 mn = h->tree.q.rootBox0, mx = h->tree.q.rootBox1;
    double L[3] = {1e300, 1e300, 1e300}, H[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < 8; ++k) {
        double p[3] = {(k & 1) ? mx.x : mn.x, (k & 2) ? mx.y : mn.y, (k & 4) ? mx.z : mn.z};
        if (tr.hasTree) {
            double q[3];
            for (int i = 0; i < 3; ++i)
                q[i] = tr.tree.A[i][0] * p[0] + tr.tree.A[i][1] * p[1] + tr.tree.A[i][2] * p[2] + tr.tree.b[i];
            std::memcpy(p, q, sizeof(q));
        }
        if (tr.hasPoint) {
            const auto& m = tr.point.A;
            const double det = double(m[0][0]) * (double(m[1][1]) * m[2][2] - double(m[1][2]) * m[2][1]) -
                               double(m[0][1]) * (double(m[1][0]) * m[2][2] - double(m[1][2]) * m[2][0]) +
                               double(m[0][2]) * (double(m[1][0]) * m[2][1] - double(m[1][1]) * m[2][0]);
            if (!(std::fabs(det) > 0)) return false;
            const double c[3][3] = {
                {double(m[1][1]) * m[2][2] - double(m[1][2]) * m[2][1], double(m[0][2]) * m[2][1] - double(m[0][1]) * m[2][2],
                 double(m[0][1]) * m[1][2] - double(m[0][2]) * m[1][1]},
                {double(m[1][2]) * m[2][0] - double(m[1][0]) * m[2][2], double(m[0][0]) * m[2][2] - double(m[0][2]) * m[2][0],
                 double(m[0][2]) * m[1][0] - double(m[0][0]) * m[1][2]},
                {double(m[1][0]) * m[2][1] - double(m[1][1]) * m[2][0], double(m[0][1]) * m[2][0] - double(m[0][0]) * m[2][1],
                 double(m[0][0]) * m[1][1] - double(m[0][1]) * m[1][0]}};
            double d[3] = {p[0] - tr.point.b[0], p[1] - tr.point.b[1], p[2] - tr.point.b[2]}, q[3];
            for (int i = 0; i < 3; ++i) q[i] = (c[i][0] * d[0] + c[i][1] * d[1] + c[i][2] * d[2]) / det;
            std::memcpy(p, q, sizeof(q));
        }
        for (int i = 0; i < 3; ++i) {
            L[i] = std::fmin(L[i], p[i]);
            H[i] = std::fmax(H[i], p[i]);
        }
    }
    for (int i = 0; i < 3; ++i) {
        lo[i] = float(L[i]);
        hi[i] = float(H[i]);
    }
    return std::isfinite(lo[0] + lo[1] + lo[2] + hi[0] + hi[1] + hi[2]);
}

cudaError_t project(gbfwn_mesh_s* h, const float* d_pts, int64_t n, const float* objXf, const float* refXf, float up, float lo,
                    gbfwn_projection* d_out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const Transforms tr = simplify(objXf, refXf);
    const Xf px = toDevice(tr.point), tx = toDevice(tr.tree);
    const int32_t* order = nullptr;
    float blo[3], bhi[3];
    if (n >= 8192 && h->tree.nLeaves > 0 && orderBox(h, tr, blo, bhi)) {
        const size_t words = size_t(n) + size_t(mortonOrderScratch(n));
        cudaError_t e = h->ensure(&h->sortBuf, &h->sortCap, words * sizeof(int32_t));
        if (e) return e;
        int32_t* buf = static_cast<int32_t*>(h->sortBuf);
        if ((e = mortonOrder(d_pts, n, blo, bhi, buf, buf + n, s))) return e;
        order = buf;
    }
    return launchProject(h->tree.q, d_pts, n, tr.hasPoint ? &px : nullptr, tr.hasTree ? &tx : nullptr, up, lo, h->precise,
                         reinterpret_cast<float4*>(d_out), h->scratch, s, order);
}

bool validXf(const float* x) {
    if (!x) return true;
    for (int i = 0; i < 12; ++i)
        if (!std::isfinite(x[i])) return false;
    return true;
}

}  // namespace

GBFWN_API int gbfwn_find_projections_dev(gbfwn_handle h, const float* d_pts, int64_t n, const float* objXf,
                                         const float* refXf, float upDistLimitSq, float loDistLimitSq,
                                         gbfwn_projection* d_out, void* stream) {
    if (!h || n < 0 || (n > 0 && (!d_pts || !d_out)) || !validXf(objXf) || !validXf(refXf))
        return fail(GBFWN_INVALID, "gbfwn_find_projections_dev: bad arguments");
    if ((reinterpret_cast<uintptr_t>(d_out) & 15) != 0)
        return fail(GBFWN_INVALID, "gbfwn_find_projections_dev: output must be 16-byte aligned");
    DeviceGuard g(h->device);
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    const cudaError_t e = project(h, d_pts, n, objXf, refXf, upDistLimitSq, loDistLimitSq, d_out, s);
    return e ? cudaFail(e, "gbfwn_find_projections_dev") : GBFWN_OK;
}

GBFWN_API int gbfwn_find_projections(gbfwn_handle h, const float* pts, int64_t n, const float* objXf, const float* refXf,
                                     float upDistLimitSq, float loDistLimitSq, gbfwn_projection* out,
                                     gbfwn_progress_cb cb, void* user) {
    const char* what = "gbfwn_find_projections";
    if (!h || n < 0 || (n > 0 && (!pts || !out)) || !validXf(objXf) || !validXf(refXf))
        return fail(GBFWN_INVALID, "gbfwn_find_projections: bad arguments");
    if (cb && cb(0.f, user) == 0) return fail(GBFWN_CANCELLED, "operation canceled");
    std::lock_guard<std::mutex> lk(h->mu);
    DeviceGuard g(h->device);
    if (n > 0) {
        cudaError_t e = h->ensure(&h->inBuf, &h->inCap, sizeof(float) * 3 * size_t(n));
        if (!e) e = h->ensure(&h->outBuf, &h->outCap, sizeof(gbfwn_projection) * size_t(n));
        if (!e) e = h->resetStatus(h->stream);
        if (!e) e = cudaMemcpyAsync(h->inBuf, pts, sizeof(float) * 3 * size_t(n), cudaMemcpyHostToDevice, h->stream);
        if (!e)
            e = project(h, static_cast<const float*>(h->inBuf), n, objXf, refXf, upDistLimitSq, loDistLimitSq,
                        static_cast<gbfwn_projection*>(h->outBuf), h->stream);
        if (!e) e = cudaMemcpyAsync(out, h->outBuf, sizeof(gbfwn_projection) * size_t(n), cudaMemcpyDeviceToHost, h->stream);
        if (!e) e = cudaStreamSynchronize(h->stream);
        if (e) return cudaFail(e, what);
        const int st = h->checkStatus();
        if (st) return st;
    }
    if (cb && cb(1.f, user) == 0) return fail(GBFWN_CANCELLED, "operation canceled");
    return GBFWN_OK;
}

GBFWN_API size_t gbfwn_projections_heap_bytes(int64_t n) {
    if (n <= 0) return 0;
    const size_t order = n >= 8192 ? size_t(n + mortonOrderScratch(n)) * sizeof(int32_t) : 0;
    return size_t(n) * (sizeof(float) * 3 + sizeof(gbfwn_projection)) + order;
}
