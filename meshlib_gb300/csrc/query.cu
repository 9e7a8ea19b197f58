// Winding-number and closest-point traversals (the per-voxel hot loops).
//
// Reference semantics (paths inside the MeshLib project):
//   winding number  MRMesh/MRDipole.cpp:94-128 (+ MRMesh/MRDipole.h:18-27, MRDipole.cpp:81-92):
//     DFS from the root; a node whose dipole is far from q (|pos - q|^2 > beta^2 * rr) contributes
//     dot(pos - q, dirArea) / |pos - q|^3 and is not opened; a near leaf contributes the exact
//     triangle solid angle; sum / (4 pi).
//   closest point   MRMesh/MRMeshProject.cpp:13-104: near-first DFS over box distances, pruning
//     boxes not closer than the best distance so far, leaf = point-triangle projection, stop once
//     the best distance is <= minDistSq.  The result is the minimum over triangles, whatever bounds
//     prune the search, so long as they never exceed the true distance: here every child carries an
//     oriented box in the frame of its area-weighted normal, which bounds a surface patch far more
//     tightly than the reference's axis-aligned box (a tilted patch's axis-aligned box sticks out
//     towards the query by up to the patch size), so far fewer nodes and triangles are visited.
//   signed distance MRMesh/MRFastWindingNumber.cpp:69-94, MRCuda/MRCudaFastWindingNumber.cu:205-243.
//
// GB300 design: one warp = one packet of 32 neighbouring queries (a 4x4x2 voxel tile for grids).
// The warp walks the UNION of the 32 per-query traversals once: a stack entry is (node, lane mask
// of the queries that still need this node), kept in registers with one entry per lane and
// moved with shuffles; node records are read once per warp (all lanes read the same address, so
// each 16-byte load is a broadcast).  Every query still makes exactly its own per-node decisions,
// so the set of dipole terms and exact solid angles summed for a query is the reference's set.
// Work is handed out by a persistent grid pulling tiles from an atomic ticket counter.
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "common.cuh"

namespace gbfwn {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int kStackDepth = 32;  // the reference's InplaceStack<..., 32>; a median-split tree of
                                 // n <= 2^31 leaves never needs more

__device__ __forceinline__ float4 ld4(const float4* p) { return __ldg(p); }

// ---- reference arithmetic helpers (no FMA contraction where decisions depend on the bits)
__device__ __forceinline__ float dot3rn(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// voxel centre: A * (x, y, z) + b, each row a left-to-right dot (MRMesh/MRMatrix3.h:127-130)
__device__ __forceinline__ float3 xfPoint(const Xf& xf, int x, int y, int z) {
    const float fx = float(x), fy = float(y), fz = float(z);
    return make_float3(__fadd_rn(dot3rn(xf.a[0], xf.a[1], xf.a[2], fx, fy, fz), xf.b[0]),
                       __fadd_rn(dot3rn(xf.a[3], xf.a[4], xf.a[5], fx, fy, fz), xf.b[1]),
                       __fadd_rn(dot3rn(xf.a[6], xf.a[7], xf.a[8], fx, fy, fz), xf.b[2]));
}

// Summation: compensated (Kahan) in precise mode, plain otherwise.
template <bool PRECISE> struct Acc {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v) {
        if (PRECISE) {
            const float y = __fsub_rn(v, c);
            const float t = __fadd_rn(s, y);
            c = __fsub_rn(__fsub_rn(t, s), y);
            s = t;
        } else {
            s = __fadd_rn(s, v);
        }
    }
};

// MRMesh/MRDipole.h:18-27.  Returns true (and adds the term) when the dipole is a good
// approximation for q.  The far-field test uses separately rounded operations like the reference.
template <bool PRECISE>
__device__ __forceinline__ bool dipoleTerm(const float4& p, const float4& da, const float3& q, float betaSq, Acc<PRECISE>& acc) {
    const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
    const float dd = dot3rn(dx, dy, dz, dx, dy, dz);
    if (dd <= __fmul_rn(betaSq, p.w)) return false;
    if (dd > 0.f) {
        const float num = dot3rn(dx, dy, dz, da.x, da.y, da.z);
        if (PRECISE) {
            const float r = rsqrtf(dd);
            acc.add(num * (r * r * r));
        } else {
            const float d = __fsqrt_rn(dd);
            acc.add(__fdiv_rn(num, __fmul_rn(d, dd)));
        }
    }
    return true;
}

// FP64 solid angle for near-plane queries; kept out of line so the rare path does not inflate the
// register allocation of the traversal loop.
__device__ __noinline__ float solidAngleFp64(const float3 q, const float4 A, const float4 B, const float4 C) {
    const double ax = double(A.x) - q.x, ay = double(A.y) - q.y, az = double(A.z) - q.z;
    const double bx = double(B.x) - q.x, by = double(B.y) - q.y, bz = double(B.z) - q.z;
    const double cx = double(C.x) - q.x, cy = double(C.y) - q.y, cz = double(C.z) - q.z;
    const double lx = sqrt(ax * ax + ay * ay + az * az);
    const double ly = sqrt(bx * bx + by * by + bz * bz);
    const double lz = sqrt(cx * cx + cy * cy + cz * cz);
    const double dd = lx * ly * lz + (ax * bx + ay * by + az * bz) * lz + (bx * cx + by * cy + bz * cz) * lx +
                      (cx * ax + cy * ay + cz * az) * ly;
    const double dt = ax * (by * cz - bz * cy) - ay * (bx * cz - bz * cx) + az * (bx * cy - by * cx);
    return float(2.0 * atan2(dt, dd));
}

// MRMesh/MRDipole.cpp:81-92: 2 * atan2(det[a-q, b-q, c-q], den) (Van Oosterom-Strackee).  In
// precise mode a query within a few ulps of the triangle plane (|det| small against the product of
// the three lengths, where the FP32 sign of det is not reliable) is re-evaluated in FP64.
template <bool PRECISE>
__device__ __forceinline__ float solidAngle(const float3& q, const float4& A, const float4& B, const float4& C) {
    const float mxx = A.x - q.x, mxy = A.y - q.y, mxz = A.z - q.z;
    const float myx = B.x - q.x, myy = B.y - q.y, myz = B.z - q.z;
    const float mzx = C.x - q.x, mzy = C.y - q.y, mzz = C.z - q.z;
    const float x = __fsqrt_rn(dot3rn(mxx, mxy, mxz, mxx, mxy, mxz));
    const float y = __fsqrt_rn(dot3rn(myx, myy, myz, myx, myy, myz));
    const float z = __fsqrt_rn(dot3rn(mzx, mzy, mzz, mzx, mzy, mzz));
    const float xyz = __fmul_rn(__fmul_rn(x, y), z);
    const float den = __fadd_rn(__fadd_rn(__fadd_rn(xyz, __fmul_rn(dot3rn(mxx, mxy, mxz, myx, myy, myz), z)),
                                          __fmul_rn(dot3rn(myx, myy, myz, mzx, mzy, mzz), x)),
                                __fmul_rn(dot3rn(mzx, mzy, mzz, mxx, mxy, mxz), y));
    const float det = __fadd_rn(__fsub_rn(__fmul_rn(mxx, __fsub_rn(__fmul_rn(myy, mzz), __fmul_rn(myz, mzy))),
                                          __fmul_rn(mxy, __fsub_rn(__fmul_rn(myx, mzz), __fmul_rn(myz, mzx)))),
                                __fmul_rn(mxz, __fsub_rn(__fmul_rn(myx, mzy), __fmul_rn(myy, mzx))));
    if (PRECISE && fabsf(det) <= 1e-5f * xyz) return solidAngleFp64(q, A, B, C);
    return 2.f * atan2f(det, den);
}

// ------------------------------------------------------------------ winding number (packet DFS)
// Lane-distributed stack: entry k lives in lane k's (stNode, stMask).
struct WarpStack {
    int node = 0;
    unsigned mask = 0;
    int sp = 0;  // warp-uniform
    __device__ __forceinline__ bool push(int lane, int n, unsigned m) {
        if (sp >= kStackDepth) return false;
        if (lane == sp) {
            node = n;
            mask = m;
        }
        ++sp;
        return true;
    }
    __device__ __forceinline__ void pop(int& n, unsigned& m) {
        --sp;
        n = __shfl_sync(FULL, node, sp);
        m = __shfl_sync(FULL, mask, sp);
    }
};

template <bool PRECISE>
__device__ __forceinline__ void leafSolidAngle(const QueryTree& t, int slot, const float3& q, bool need, int skipSlot,
                                               Acc<PRECISE>& acc) {
    const float4* tr = t.tri + 3 * int64_t(slot);
    const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
    if (need && slot != skipSlot) acc.add(solidAngle<PRECISE>(q, A, B, C));
}

// Winding number of q (lanes with active == false only ride along).  Returns sum / (4 pi).
template <bool PRECISE>
__device__ float fwnPacket(const QueryTree& t, const float3& q, bool active, float betaSq, int skipSlot, unsigned* status) {
    const int lane = threadIdx.x & 31;
    Acc<PRECISE> acc;
    if (__ballot_sync(FULL, active) == 0 || t.nLeaves == 0) return 0.f;
    bool need = active && !dipoleTerm<PRECISE>(t.rootDip0, t.rootDip1, q, betaSq, acc);
    const unsigned rootNeed = __ballot_sync(FULL, need);
    WarpStack st;
    if (rootNeed) {
        const int rootLink = __float_as_int(t.rootDip1.w);
        if (rootLink < 0)
            leafSolidAngle<PRECISE>(t, ~rootLink, q, need, skipSlot, acc);
        else
            st.push(lane, rootLink, rootNeed);
    }
    bool overflow = false;
    while (st.sp > 0) {
        int node;
        unsigned m;
        st.pop(node, m);
        const float4* rec = t.dip + 4 * int64_t(node);
        const float4 l0 = ld4(rec), l1 = ld4(rec + 1), r0 = ld4(rec + 2), r1 = ld4(rec + 3);
        const bool mine = (m >> lane) & 1u;
        bool nl = false, nr = false;
        if (mine) {
            nl = !dipoleTerm<PRECISE>(l0, l1, q, betaSq, acc);
            nr = !dipoleTerm<PRECISE>(r0, r1, q, betaSq, acc);
        }
        const unsigned ml = __ballot_sync(FULL, nl), mr = __ballot_sync(FULL, nr);
        const int ll = __float_as_int(l1.w), rl = __float_as_int(r1.w);
        // right subtree below left on the stack, so the left subtree is summed first (reference order)
        if (mr) {
            if (rl < 0)
                leafSolidAngle<PRECISE>(t, ~rl, q, nr, skipSlot, acc);
            else if (!st.push(lane, rl, mr))
                overflow = true;
        }
        if (ml) {
            if (ll < 0)
                leafSolidAngle<PRECISE>(t, ~ll, q, nl, skipSlot, acc);
            else if (!st.push(lane, ll, ml))
                overflow = true;
        }
        if (overflow) break;
    }
    if (overflow && lane == 0) atomicOr(status, kStatusStackOverflow);
    const float INV_4PI = 1.0f / (4 * 3.14159265358979f);
    return __fmul_rn(INV_4PI, PRECISE ? __fsub_rn(acc.s, acc.c) : acc.s);
}

// Winding numbers of two queries per lane in one packet walk (voxels qa and qb of the lane): the stack
// carries a lane mask per query, each query takes its own far / near decisions into its own sum in
// its own depth-first order, so each result equals fwnPacket's for that query bit for bit, while the
// records and stack steps are shared by 64 queries.
template <bool PRECISE>
__device__ void fwnPacket2(const QueryTree& t, const float3& qa, const float3& qb, bool activeA, bool activeB, float betaSq,
                           unsigned* status, float* wa, float* wb) {
    const int lane = threadIdx.x & 31;
    Acc<PRECISE> accA, accB;
    const float INV_4PI = 1.0f / (4 * 3.14159265358979f);
    *wa = *wb = 0.f;
    if (__ballot_sync(FULL, activeA || activeB) == 0 || t.nLeaves == 0) return;
    const bool needA = activeA && !dipoleTerm<PRECISE>(t.rootDip0, t.rootDip1, qa, betaSq, accA);
    const bool needB = activeB && !dipoleTerm<PRECISE>(t.rootDip0, t.rootDip1, qb, betaSq, accB);
    const unsigned rootA = __ballot_sync(FULL, needA), rootB = __ballot_sync(FULL, needB);
    // stack: node and the two masks, one entry per lane
    int stNode = 0;
    unsigned stA = 0, stB = 0;
    int sp = 0;
    if (rootA | rootB) {
        const int rootLink = __float_as_int(t.rootDip1.w);
        if (rootLink < 0) {
            leafSolidAngle<PRECISE>(t, ~rootLink, qa, needA, -1, accA);
            leafSolidAngle<PRECISE>(t, ~rootLink, qb, needB, -1, accB);
        } else {
            if (lane == 0) {
                stNode = rootLink;
                stA = rootA;
                stB = rootB;
            }
            sp = 1;
        }
    }
    bool overflow = false;
    while (sp > 0) {
        --sp;
        const int node = __shfl_sync(FULL, stNode, sp);
        const unsigned mA = __shfl_sync(FULL, stA, sp), mB = __shfl_sync(FULL, stB, sp);
        const float4* rec = t.dip + 4 * int64_t(node);
        const float4 l0 = ld4(rec), l1 = ld4(rec + 1), r0 = ld4(rec + 2), r1 = ld4(rec + 3);
        bool nlA = false, nrA = false, nlB = false, nrB = false;
        if ((mA >> lane) & 1u) {
            nlA = !dipoleTerm<PRECISE>(l0, l1, qa, betaSq, accA);
            nrA = !dipoleTerm<PRECISE>(r0, r1, qa, betaSq, accA);
        }
        if ((mB >> lane) & 1u) {
            nlB = !dipoleTerm<PRECISE>(l0, l1, qb, betaSq, accB);
            nrB = !dipoleTerm<PRECISE>(r0, r1, qb, betaSq, accB);
        }
        const unsigned mlA = __ballot_sync(FULL, nlA), mrA = __ballot_sync(FULL, nrA);
        const unsigned mlB = __ballot_sync(FULL, nlB), mrB = __ballot_sync(FULL, nrB);
        const int ll = __float_as_int(l1.w), rl = __float_as_int(r1.w);
        // right subtree below left on the stack, so the left subtree is summed first (as fwnPacket)
        if (mrA | mrB) {
            if (rl < 0) {
                leafSolidAngle<PRECISE>(t, ~rl, qa, nrA, -1, accA);
                leafSolidAngle<PRECISE>(t, ~rl, qb, nrB, -1, accB);
            } else if (sp >= kStackDepth) {
                overflow = true;
            } else {
                if (lane == sp) {
                    stNode = rl;
                    stA = mrA;
                    stB = mrB;
                }
                ++sp;
            }
        }
        if (mlA | mlB) {
            if (ll < 0) {
                leafSolidAngle<PRECISE>(t, ~ll, qa, nlA, -1, accA);
                leafSolidAngle<PRECISE>(t, ~ll, qb, nlB, -1, accB);
            } else if (sp >= kStackDepth) {
                overflow = true;
            } else {
                if (lane == sp) {
                    stNode = ll;
                    stA = mlA;
                    stB = mlB;
                }
                ++sp;
            }
        }
        if (overflow) break;
    }
    if (overflow && lane == 0) atomicOr(status, kStatusStackOverflow);
    *wa = __fmul_rn(INV_4PI, PRECISE ? __fsub_rn(accA.s, accA.c) : accA.s);
    *wb = __fmul_rn(INV_4PI, PRECISE ? __fsub_rn(accB.s, accB.c) : accB.s);
}

// ------------------------------------------------------------------ closest point (packet DFS)
__device__ __forceinline__ float boxDistSq(const float4& mn, const float4& mx, const float3& p) {
    // MRMesh/MRBox.h:207-220 (reference arithmetic)
    float r = 0.f, d;
    if (p.x < mn.x) { d = p.x - mn.x; r = __fadd_rn(r, __fmul_rn(d, d)); }
    else if (p.x > mx.x) { d = p.x - mx.x; r = __fadd_rn(r, __fmul_rn(d, d)); }
    if (p.y < mn.y) { d = p.y - mn.y; r = __fadd_rn(r, __fmul_rn(d, d)); }
    else if (p.y > mx.y) { d = p.y - mx.y; r = __fadd_rn(r, __fmul_rn(d, d)); }
    if (p.z < mn.z) { d = p.z - mn.z; r = __fadd_rn(r, __fmul_rn(d, d)); }
    else if (p.z > mx.z) { d = p.z - mx.z; r = __fadd_rn(r, __fmul_rn(d, d)); }
    return r;
}

// A closest-point record (layout in common.cuh): the node's frame and both children's boxes in it.
struct CpRecord {
    float3 t, u, n;
    float3 cl, el, cr, er;
    int ll, rl;
};
__device__ __forceinline__ CpRecord loadCp(const float4* rec) {
    const float4 r0 = ld4(rec), r1 = ld4(rec + 1), r2 = ld4(rec + 2), r3 = ld4(rec + 3), r4 = ld4(rec + 4), r5 = ld4(rec + 5);
    CpRecord c;
    c.t = make_float3(r0.x, r0.y, r0.z);
    c.u = make_float3(r0.w, r1.x, r1.y);
    c.n = make_float3(r1.z, r1.w, r2.x);
    c.cl = make_float3(r2.y, r2.z, r2.w);
    c.el = make_float3(r3.x, r3.y, r3.z);
    c.cr = make_float3(r4.x, r4.y, r4.z);
    c.er = make_float3(r4.w, r5.x, r5.y);
    c.ll = __float_as_int(r3.w);
    c.rl = __float_as_int(r5.z);
    return c;
}

// Squared distance from the point with frame coordinates x to the box (centre c, half extents e)
// in that frame: a lower bound of the distance to any triangle of the subtree (the extents carry a
// rounding margin).
__device__ __forceinline__ float frameBoxDistSq(const float3& x, const float3& c, const float3& e) {
    const float dt = fmaxf(fabsf(x.x - c.x) - e.x, 0.f), du = fmaxf(fabsf(x.y - c.y) - e.y, 0.f),
                dn = fmaxf(fabsf(x.z - c.z) - e.z, 0.f);
    return fmaf(dt, dt, fmaf(du, du, dn * dn));
}

__device__ __forceinline__ float3 toFrame(const CpRecord& r, const float3& p) {
    return make_float3(fmaf(r.t.x, p.x, fmaf(r.t.y, p.y, r.t.z * p.z)), fmaf(r.u.x, p.x, fmaf(r.u.y, p.y, r.u.z * p.z)),
                       fmaf(r.n.x, p.x, fmaf(r.n.y, p.y, r.n.z * p.z)));
}

// Affine map of a mesh-space point (rows of A, left-to-right dots, then + b: MRMesh/MRMatrix3.h:127-130).
__device__ __forceinline__ float3 xfApply(const Xf& xf, float x, float y, float z) {
    return make_float3(__fadd_rn(dot3rn(xf.a[0], xf.a[1], xf.a[2], x, y, z), xf.b[0]),
                       __fadd_rn(dot3rn(xf.a[3], xf.a[4], xf.a[5], x, y, z), xf.b[1]),
                       __fadd_rn(dot3rn(xf.a[6], xf.a[7], xf.a[8], x, y, z), xf.b[2]));
}

// Squared distance from p to the axis-aligned box around the image of a mesh-space box (centre c,
// half extents h along the orthonormal axes d0, d1, d2) under the affine map xf: a lower bound of
// the distance to anything inside that box once mapped.  The half extents get a relative margin
// for the rounding of the mapped triangle vertices.
__device__ __forceinline__ float mappedBoxDistSq(const Xf& xf, const float3& c, const float3& d0, const float3& d1,
                                                 const float3& d2, const float3& h, const float3& p) {
    float r = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a0 = xf.a[3 * k], a1 = xf.a[3 * k + 1], a2 = xf.a[3 * k + 2];
        const float ck = fmaf(a0, c.x, fmaf(a1, c.y, fmaf(a2, c.z, xf.b[k])));
        float hk = fabsf(fmaf(a0, d0.x, fmaf(a1, d0.y, a2 * d0.z))) * h.x + fabsf(fmaf(a0, d1.x, fmaf(a1, d1.y, a2 * d1.z))) * h.y +
                   fabsf(fmaf(a0, d2.x, fmaf(a1, d2.y, a2 * d2.z))) * h.z;
        hk += 4e-6f * (fabsf(ck) + hk + fabsf(xf.b[k])) + 1e-30f;
        const float pk = k == 0 ? p.x : k == 1 ? p.y : p.z;
        const float dk = fmaxf(fabsf(pk - ck) - hk, 0.f);
        r = fmaf(dk, dk, r);
    }
    return r;
}

// a child's box of a record seen through the affine map xf
__device__ __forceinline__ float frameBoxDistSqXf(const Xf& xf, const CpRecord& r, const float3& c, const float3& e,
                                                 const float3& p) {
    const float3 ctr = make_float3(fmaf(c.x, r.t.x, fmaf(c.y, r.u.x, c.z * r.n.x)), fmaf(c.x, r.t.y, fmaf(c.y, r.u.y, c.z * r.n.y)),
                                   fmaf(c.x, r.t.z, fmaf(c.y, r.u.z, c.z * r.n.z)));
    return mappedBoxDistSq(xf, ctr, r.t, r.u, r.n, e, p);
}

// root box (axis-aligned, min/max) seen through xf
__device__ __forceinline__ float rootBoxDistSqXf(const Xf& xf, const float4& mn, const float4& mx, const float3& p) {
    const float3 c = make_float3(0.5f * (mn.x + mx.x), 0.5f * (mn.y + mx.y), 0.5f * (mn.z + mx.z));
    const float3 h = make_float3(0.5f * (mx.x - mn.x), 0.5f * (mx.y - mn.y), 0.5f * (mx.z - mn.z));
    const float3 h2 = make_float3(h.x + 1e-6f * (fabsf(c.x) + h.x), h.y + 1e-6f * (fabsf(c.y) + h.y), h.z + 1e-6f * (fabsf(c.z) + h.z));
    return mappedBoxDistSq(xf, c, make_float3(1.f, 0.f, 0.f), make_float3(0.f, 1.f, 0.f), make_float3(0.f, 0.f, 1.f), h2, p);
}

template <typename T> struct V3T {
    T x, y, z;
};
template <typename T> __device__ __forceinline__ V3T<T> vsub(V3T<T> a, V3T<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> __device__ __forceinline__ T vdot(V3T<T> a, V3T<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> __device__ __forceinline__ V3T<T> vmad(V3T<T> a, T s, V3T<T> b) { return {a.x + s * b.x, a.y + s * b.y, a.z + s * b.z}; }

// MRMesh/MRClosestPointInTriangle.h:28-91 (Voronoi-region projection).
template <typename T> __device__ __forceinline__ V3T<T> closestPoint(V3T<T> p, V3T<T> a, V3T<T> b, V3T<T> c) {
    const V3T<T> ab = vsub(b, a), ac = vsub(c, a), ap = vsub(p, a);
    const T d1 = vdot(ab, ap), d2 = vdot(ac, ap);
    if (d1 <= 0 && d2 <= 0) return a;
    const V3T<T> bp = vsub(p, b);
    const T d3 = vdot(ab, bp), d4 = vdot(ac, bp);
    if (d3 >= 0 && d4 <= d3) return b;
    const V3T<T> cp = vsub(p, c);
    const T d5 = vdot(ab, cp), d6 = vdot(ac, cp);
    if (d6 >= 0 && d5 <= d6) return c;
    const T vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) return vmad(a, d1 / (d1 - d3), ab);
    const T vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d6 <= 0 && d2 >= 0) return vmad(a, d2 / (d2 - d6), ac);
    const T va = d3 * d6 - d5 * d4;
    if (va <= 0) {
        if (d4 < d3) return b;
        if (d5 < d6) return c;
        return vmad(b, (d4 - d3) / ((d4 - d3) + (d5 - d6)), vsub(c, b));
    }
    const T denom = T(1) / (va + vb + vc);
    return vmad(vmad(a, vb * denom, ab), vc * denom, ac);
}

// FP64 projection (as the reference CPU does for every leaf, MRMesh/MRMeshProject.cpp:66-72): the
// projection is rounded to float and the distance measured in float.  Out of line: rare path.
__device__ __noinline__ float triDistSqFp64(const float3 p, const float4 A, const float4 B, const float4 C) {
    const V3T<double> pd{p.x, p.y, p.z}, ad{A.x, A.y, A.z}, bd{B.x, B.y, B.z}, cd{C.x, C.y, C.z};
    const V3T<double> q = closestPoint<double>(pd, ad, bd, cd);
    const float qx = float(q.x) - p.x, qy = float(q.y) - p.y, qz = float(q.z) - p.z;
    return dot3rn(qx, qy, qz, qx, qy, qz);
}

// Squared distance from p to a triangle (a leaf record: C.w holds its nearPlaneLevel).  FP32
// projection; in precise mode a query that lands within ~1e-4 triangle edge lengths of the triangle
// (below C.w) is re-projected in FP64.
template <bool PRECISE>
__device__ __forceinline__ float triDistSq(const float3& p, const float4& A, const float4& B, const float4& C) {
    const V3T<float> pf{p.x, p.y, p.z}, af{A.x, A.y, A.z}, bf{B.x, B.y, B.z}, cf{C.x, C.y, C.z};
    const V3T<float> pr = closestPoint<float>(pf, af, bf, cf);
    const V3T<float> d = vsub(pr, pf);
    float ds = dot3rn(d.x, d.y, d.z, d.x, d.y, d.z);
    if (PRECISE && ds < C.w) ds = triDistSqFp64(p, A, B, C);
    return ds;
}

__device__ __forceinline__ float4 xf4(const Xf* xf, const float4& v) {
    const float3 r = xfApply(*xf, v.x, v.y, v.z);
    return make_float4(r.x, r.y, r.z, v.w);
}
// A leaf triangle seen through the affine map *xf, its near-plane level recomputed for the mapped one.
__device__ __forceinline__ void xfTri(const Xf* xf, float4& A, float4& B, float4& C) {
    A = xf4(xf, A);
    B = xf4(xf, B);
    C = xf4(xf, C);
    C.w = nearPlaneLevel(A, B, C);
}

// TRACK: remember the leaf slot of the best triangle in *best; TREEXF: the mesh is seen through
// the affine map *txf (its triangle vertices are mapped before the distance, as the reference does
// for a non-rigid tree transform, MRMesh/MRMeshProject.cpp:57-63).
template <bool PRECISE, bool TRACK = false, bool TREEXF = false>
__device__ __forceinline__ void leafDist(const QueryTree& t, int slot, const float3& q, bool go, float& resSq, bool& done,
                                         float loSq, int* best = nullptr, const Xf* txf = nullptr) {
    const float4* tr = t.tri + 3 * int64_t(slot);
    float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
    if (go) {
        if (TREEXF) {
            xfTri(txf, A, B, C);
        }
        const float ds = triDistSq<PRECISE>(q, A, B, C);
        if (ds < resSq) {
            resSq = ds;
            if (TRACK) *best = slot;
            if (ds <= loSq) done = true;
        }
    }
}

// Closest squared distance from q to the mesh, starting from the bound upSq (the reference's
// maxDistSq) and stopping once <= loSq; returns upSq when nothing is closer.
template <bool PRECISE, bool TRACK = false, bool TREEXF = false>
__device__ float cpPacket(const QueryTree& t, const float3& q, bool active, float upSq, float loSq, unsigned* status,
                          int* best = nullptr, const Xf* txf = nullptr) {
    const int lane = threadIdx.x & 31;
    float resSq = upSq;
    bool done = !active;
    if (__ballot_sync(FULL, active) == 0 || t.nLeaves == 0) return resSq;
    const float rootD = TREEXF ? rootBoxDistSqXf(*txf, t.rootBox0, t.rootBox1, q) : boxDistSq(t.rootBox0, t.rootBox1, q);
    const bool inRoot = active && rootD < resSq;
    const unsigned m0 = __ballot_sync(FULL, inRoot);
    if (!m0) return resSq;
    const int rootLink = __float_as_int(t.rootBox0.w);
    if (rootLink < 0) {
        leafDist<PRECISE, TRACK, TREEXF>(t, ~rootLink, q, inRoot, resSq, done, loSq, best, txf);
        return resSq;
    }
    WarpStack st;
    st.push(lane, rootLink, m0);
    bool overflow = false;
    while (st.sp > 0) {
        int node;
        unsigned m;
        st.pop(node, m);
        const CpRecord rec = loadCp(t.cp + 6 * int64_t(node));
        const bool mine = ((m >> lane) & 1u) && !done;
        const int ll = rec.ll, rl = rec.rl;
        float dl, dr;
        if (TREEXF) {
            dl = frameBoxDistSqXf(*txf, rec, rec.cl, rec.el, q);
            dr = frameBoxDistSqXf(*txf, rec, rec.cr, rec.er, q);
        } else {
            const float3 x = toFrame(rec, q);  // one projection for both children
            dl = frameBoxDistSq(x, rec.cl, rec.el);
            dr = frameBoxDistSq(x, rec.cr, rec.er);
        }
        if (!mine) {
            dl = FLT_MAX;
            dr = FLT_MAX;
        }
        const bool gl = mine && dl < resSq, gr = mine && dr < resSq;
        const unsigned ml = __ballot_sync(FULL, gl), mr = __ballot_sync(FULL, gr);
        if ((ml | mr) == 0) continue;
        // near first: the child more queries prefer (ties: right first, as the reference does
        // when the two distances are equal)
        const unsigned preferL = __ballot_sync(FULL, gl && gr ? dl < dr : gl);
        const unsigned both = ml | mr;
        const bool leftFirst = 2 * __popc(preferL & both) > __popc(both);
        // leaves are evaluated at once (near one first), inner children pushed far-then-near
        const int nearLink = leftFirst ? ll : rl, farLink = leftFirst ? rl : ll;
        const unsigned nearM = leftFirst ? ml : mr, farM = leftFirst ? mr : ml;
        const float nearD = leftFirst ? dl : dr, farD = leftFirst ? dr : dl;
        const bool nearGo = leftFirst ? gl : gr, farGo = leftFirst ? gr : gl;
        if (nearM && nearLink < 0) leafDist<PRECISE, TRACK, TREEXF>(t, ~nearLink, q, nearGo && !done, resSq, done, loSq, best, txf);
        if (farM && farLink < 0)
            leafDist<PRECISE, TRACK, TREEXF>(t, ~farLink, q, farGo && !done && farD < resSq, resSq, done, loSq, best, txf);
        if (farM && farLink >= 0 && !st.push(lane, farLink, farM)) overflow = true;
        if (nearM && nearLink >= 0 && !st.push(lane, nearLink, nearM)) overflow = true;
        (void)nearD;
        if (overflow) break;
    }
    if (overflow && lane == 0) atomicOr(status, kStatusStackOverflow);
    return resSq;
}

// Per warp of a paired walk, the lanes whose lower / upper query came within a triangle's near-plane
// level (kept in shared memory: set rarely, and no register carries them through the walk).
__shared__ uint32_t sPairFix[8][2];

// One leaf triangle for the two queries of a lane (loaded once), in FP32; FLAG: a query that comes
// within the triangle's near-plane level (where the precise distance would be re-evaluated in FP64)
// sets its lane's bit in sPairFix, and the caller evaluates that query again with the precise walk.
template <bool FLAG>
__device__ __forceinline__ void leafDist2(const QueryTree& t, int slot, const float3& qa, const float3& qb, bool goA, bool goB,
                                          float& resA, float& resB, int& bestA, int& bestB, bool& doneA, bool& doneB) {
    const float4* tr = t.tri + 3 * int64_t(slot);
    const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
    if (goA) {
        const float ds = triDistSq<false>(qa, A, B, C);
        if (FLAG && ds < C.w) atomicOr(&sPairFix[threadIdx.x >> 5][0], 1u << (threadIdx.x & 31));
        if (ds < resA) {
            resA = ds;
            bestA = slot;
            if (ds <= 0.f) doneA = true;
        }
    }
    if (goB) {
        const float ds = triDistSq<false>(qb, A, B, C);
        if (FLAG && ds < C.w) atomicOr(&sPairFix[threadIdx.x >> 5][1], 1u << (threadIdx.x & 31));
        if (ds < resB) {
            resB = ds;
            bestB = slot;
            if (ds <= 0.f) doneB = true;
        }
    }
}

// Two queries per lane in one packet walk (voxels qa and qb of the lane): a node is opened when either
// query of any lane may hold a closer triangle, each query keeps its own bound and prunes its own
// leaves, so each result is its exact minimum, as with cpPacket (no early stop: loSq = 0).  FP32
// triangle distances; FLAG as leafDist2.  vertical: qb lies straight above qa (same x and y), and its
// frame coordinates follow from qa's.
template <bool FLAG>
__device__ void cpPacket2(const QueryTree& t, const float3& qa, const float3& qb, bool activeA, bool activeB, float& resA,
                          float& resB, int& bestA, int& bestB, unsigned* status, bool vertical = true) {
    const float dzB = qb.z - qa.z;  // vertical: qb = qa + (0, 0, dzB), the same x and y (a vertical grid column)
    const int lane = threadIdx.x & 31;
    if (t.nLeaves == 0) return;
    const bool inA = activeA && boxDistSq(t.rootBox0, t.rootBox1, qa) < resA;
    const bool inB = activeB && boxDistSq(t.rootBox0, t.rootBox1, qb) < resB;
    const unsigned m0 = __ballot_sync(FULL, inA || inB);
    if (!m0) return;
    const int rootLink = __float_as_int(t.rootBox0.w);
    bool doneA = !activeA, doneB = !activeB;
    if (rootLink < 0) {
        leafDist2<FLAG>(t, ~rootLink, qa, qb, inA, inB, resA, resB, bestA, bestB, doneA, doneB);
        return;
    }
    WarpStack st;
    st.push(lane, rootLink, m0);
    bool overflow = false;
    while (st.sp > 0) {
        int node;
        unsigned m;
        st.pop(node, m);
        const CpRecord rec = loadCp(t.cp + 6 * int64_t(node));
        const bool mine = (m >> lane) & 1u;
        // qb lies straight above qa (grids with a vertical z axis), so its frame coordinates follow
        // from qa's by the frame's z column: three FMAs instead of nine (the boxes' rounding margin,
        // 2e-6 of the coordinates, covers the few ulps this differs from projecting qb itself)
        const float3 xa = toFrame(rec, qa);
        const float3 xb = vertical ? make_float3(fmaf(dzB, rec.t.z, xa.x), fmaf(dzB, rec.u.z, xa.y), fmaf(dzB, rec.n.z, xa.z))
                                   : toFrame(rec, qb);
        float dla = frameBoxDistSq(xa, rec.cl, rec.el), dra = frameBoxDistSq(xa, rec.cr, rec.er);
        float dlb = frameBoxDistSq(xb, rec.cl, rec.el), drb = frameBoxDistSq(xb, rec.cr, rec.er);
        const bool gla = mine && !doneA && dla < resA, gra = mine && !doneA && dra < resA;
        const bool glb = mine && !doneB && dlb < resB, grb = mine && !doneB && drb < resB;
        const bool gl = gla || glb, gr = gra || grb;
        const unsigned ml = __ballot_sync(FULL, gl), mr = __ballot_sync(FULL, gr);
        if ((ml | mr) == 0) continue;
        const float dl = fminf(gla ? dla : FLT_MAX, glb ? dlb : FLT_MAX), dr = fminf(gra ? dra : FLT_MAX, grb ? drb : FLT_MAX);
        const unsigned preferL = __ballot_sync(FULL, gl && gr ? dl < dr : gl);
        const unsigned both = ml | mr;
        const bool leftFirst = 2 * __popc(preferL & both) > __popc(both);
        const int nearLink = leftFirst ? rec.ll : rec.rl, farLink = leftFirst ? rec.rl : rec.ll;
        const unsigned nearM = leftFirst ? ml : mr, farM = leftFirst ? mr : ml;
        const bool nearA = leftFirst ? gla : gra, nearB = leftFirst ? glb : grb;
        const bool farA = leftFirst ? gra : gla, farB = leftFirst ? grb : glb;
        const float farDA = leftFirst ? dra : dla, farDB = leftFirst ? drb : dlb;
        if (nearM && nearLink < 0)
            leafDist2<FLAG>(t, ~nearLink, qa, qb, nearA, nearB, resA, resB, bestA, bestB, doneA, doneB);
        if (farM && farLink < 0)
            leafDist2<FLAG>(t, ~farLink, qa, qb, farA && !doneA && farDA < resA, farB && !doneB && farDB < resB, resA, resB, bestA,
                            bestB, doneA, doneB);
        if (farM && farLink >= 0 && !st.push(lane, farLink, farM)) overflow = true;
        if (nearM && nearLink >= 0 && !st.push(lane, nearLink, nearM)) overflow = true;
        if (overflow) break;
    }
    if (overflow && lane == 0) atomicOr(status, kStatusStackOverflow);
}

// ------------------------------------------------------------------ kernels
constexpr int kThreads = 256;
static_assert(kThreads / 32 == sizeof(sPairFix) / sizeof(sPairFix[0]), "one sPairFix row per warp");
// Resident blocks per SM of the kernels that run the closest-point walk (48 registers, a few values
// spilled): more warps hide the dependent record loads better than registers help, up to the point
// where spills take over.  Measured at 512^3 on 1.31 M triangles with the 128-byte two-frame records:
// 4 blocks (64 registers) 129 ms, 5 (48) 120 ms, 6 (40) 115 ms, 7-8 150 ms; with the 96-byte one-frame
// records: 5 blocks 108.5 ms, 6 blocks 110.0 ms, 7 blocks 144.5 ms.  The winding-number-only walks keep
// 4 (23.4 -> 25.1 ms at 6); so do self-intersections and the batched kernel, which measured slower with
// more warps.
constexpr int kDistBlocks = 5;
// Resident blocks per SM of the paired walk (two voxels per lane): 48 registers, no spills.  Measured
// at 512^3 on 1.31 M triangles: 4 blocks 69.3 ms, 5 63.6 ms, 6 68.0 ms.
constexpr int kPairBlocks = 5;
// Voxel tile of one warp.  Measured at 512^3 on 1.31 M triangles with sign reuse (the same grids for
// every shape): 4x4x2 84.2 ms, 2x4x4 88.5, 4x2x4 88.6, 8x4x1 103.1, 4x8x1 102.8.
constexpr int kTX = 4, kTY = 4, kTZ = 2;
constexpr int kLayer = kTX * kTY;         // lanes per tile layer
// an 8x8x8-voxel brick of the banded path: columns of kBrickSeg tiles, kBrickCols of them
constexpr int kBrickColsX = 8 / kTX, kBrickCols = (8 / kTX) * (8 / kTY), kBrickSeg = 8 / kTZ;
static_assert(kTX * kTY * kTZ == 32 && 8 % kTX == 0 && 8 % kTY == 0 && 8 % kTZ == 0, "tile shape");

struct TileGrid {
    int32_t tilesX, tilesY, tilesZ;
    uint32_t numTiles;
    // optional runs of 8x8x8-voxel bricks to cover instead of the whole range: (bx, by, bz0, count),
    // `count` bricks stacked from brick layer bz0 upwards; kBrickCols tile columns per run, each
    // walked through the whole run, so its state carries from brick to brick
    const int4* runs;
    // work items: columns of up to segLen tiles along z (kBrickCols per brick run)
    int32_t segLen, segsZ;
    uint32_t numItems;
    // optional hand-over between the columns of one launch (whole grids only): 2 x kLayer words per
    // work item, written when the item ends -- words [0, kLayer) the signed squared distance of each
    // top-layer voxel (negative inside, NaN when its sign is unknown), then the leaf slot closest to it
    // (-1 none) -- and read by the column above it when it starts; filled with 0xff bytes (NaN / -1)
    // before the launch, so a column that starts before the one below it has ended starts cold
    float* colState;
    // optional inside bits of every voxel of the range (signColumnsKernel's layout: one word per 32
    // voxels along x, (z - zOut, y, x / 32)); when given, the signed-distance kernel takes its signs
    // from them instead of its own walks
    const uint32_t* signBits;
    // precise paired walks: the pair steps with voxels that came within a triangle's near-plane level,
    // {item, first tile, lane mask of the lower voxels, of the upper ones}, re-walked by fixPairKernel;
    // fixList[0].x counts them (capacity fixCap entries after it)
    uint4* fixList;
    uint32_t fixCap;
};

__device__ __forceinline__ unsigned nextTicket(unsigned* counter, int lane) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(counter, 1u);
    return __shfl_sync(FULL, t, 0);
}

// Whether a signed-distance voxel may take its sign from a voxel below it (closed surfaces only):
// the exact winding number of a closed oriented surface is an integer, constant along any segment
// that does not meet the surface, and the segment between two voxel centres meets none when it is
// shorter than the lower voxel's distance to the surface.  The approximated winding numbers of both
// voxels then lie within their approximation error of the same integer, so with the threshold away
// from integers (fractional part in (0.25, 0.75)) and the dipole criterion at beta >= 2 they fall on
// the same side of it, and the sign computed below is the one the upper voxel's own winding number
// would give.
__device__ __forceinline__ bool signReuseAllowed(const QueryTree& t, const DistOpts& o) {
    const float fr = o.threshold - floorf(o.threshold);
    return t.closed != 0 && o.beta >= 2.f && fr > 0.25f && fr < 0.75f;
}

// ------------------------------------------------------------------ ray crossings (closed surfaces)
// Kahan's 2x2 determinant a*b - c*d: relative error at most 2u (Jeannerod, Louvet and Muller, 2013),
// so its sign is exact and it is 0 exactly when a*b == c*d.
__device__ __forceinline__ float det2(float a, float b, float c, float d) {
    const float w = __fmul_rn(c, d);
    const float e = fmaf(-c, d, w);
    const float f = fmaf(a, b, -w);
    return __fadd_rn(f, e);
}

// Sign of the edge function E(P, Q) = Px Qy - Py Qx of a projected edge P -> Q (coordinates relative
// to the ray's origin), exact, with E = 0 broken by simulation of simplicity: the origin moved by
// (eps, eps^2), eps -> 0, changes E by eps (Py - Qy) + eps^2 (Qx - Px).  Swapping P and Q flips the
// sign, so a ray meets exactly one of two triangles that share an edge on the same side of it, and
// both or neither of two that fold over it.  0 only for a degenerate edge.
__device__ __forceinline__ int edgeSignOf(float e, float px, float py, float qx, float qy) {
    if (e != 0.f) return e > 0.f ? 1 : -1;
    if (py != qy) return py > qy ? 1 : -1;
    if (qx != px) return qx > px ? 1 : -1;
    return 0;
}
__device__ __forceinline__ int edgeSign(float px, float py, float qx, float qy) {
    return edgeSignOf(det2(px, qy, py, qx), px, py, qx, qy);
}

// Squared distance from the origin to the segment P -> Q in the plane (a test of closeness only: fast
// division, FP32).
__device__ __forceinline__ float segDistSq0(float px, float py, float qx, float qy) {
    const float dx = qx - px, dy = qy - py;
    const float dd = fmaf(dx, dx, dy * dy);
    float s = dd > 0.f ? __fdividef(-fmaf(px, dx, py * dy), dd) : 0.f;
    s = fminf(fmaxf(s, 0.f), 1.f);
    const float rx = fmaf(s, dx, px), ry = fmaf(s, dy, py);
    return fmaf(rx, rx, ry * ry);
}

// Whether the origin lies within sqrt(epsSq) of the boundary of the projected triangle (a, b, c):
// a vertical ray through it runs through an edge or a vertex, or along a vertical triangle, where a
// point of the ray may lie on the surface without a crossing at its height.
__device__ __forceinline__ bool nearProjection(float ax, float ay, float bx, float by, float cx, float cy, float epsSq) {
    return segDistSq0(ax, ay, bx, by) <= epsSq || segDistSq0(bx, by, cx, cy) <= epsSq || segDistSq0(cx, cy, ax, ay) <= epsSq;
}

// Tolerances of the vertical-ray tests of a mesh: zTol on heights (1e-12 of the largest |z|, far above
// the FP64 heights' rounding) and epsSq on the (x, y) closeness to a triangle's boundary (4e-6 of the
// largest |x|, |y|: a few tens of FP32 ulps).
__device__ __forceinline__ double rayZTol(const QueryTree& t) {
    return 1e-12 * double(fmaxf(fabsf(t.rootBox0.z), fabsf(t.rootBox1.z)));
}
__device__ __forceinline__ float rayEpsSq(const QueryTree& t) {
    const float e = 4e-6f * fmaxf(fmaxf(fabsf(t.rootBox0.x), fabsf(t.rootBox1.x)), fmaxf(fabsf(t.rootBox0.y), fabsf(t.rootBox1.y)));
    return e * e;
}

// Signed crossing of the vertical ray from q (up: +z, else -z) with triangle ABC: the crossing's
// contribution to the winding number at q, +1 where the ray passes to the side the triangle's normal
// points to and -1 the other way (a ray from inside a closed outward-oriented surface leaves it once
// more than it enters), 0 when it misses.  The triangle is translated to the ray's origin in FP32, the
// same way in every triangle that shares a vertex, so the translated mesh is closed as well and every
// ray crosses it an exact number of times.  A crossing at the origin itself (q on the surface, where
// the winding number decides between 0 and 1 by its approximation) sets *onSurface instead, and so
// does a vertical triangle (flagged in B.w when the leaf records are packed: a projection with next
// to no area) whose z range holds q's and whose projection passes within sqrt(epsSq) of q (q may lie
// on it, and no vertical ray crosses it).
__device__ __forceinline__ int rayCross(const float3& q, const float4& A, const float4& B, const float4& C, bool up,
                                        bool* onSurface, float epsSq, float zTolF) {
    const float ax = __fsub_rn(A.x, q.x), ay = __fsub_rn(A.y, q.y), bx = __fsub_rn(B.x, q.x), by = __fsub_rn(B.y, q.y),
                cx = __fsub_rn(C.x, q.x), cy = __fsub_rn(C.y, q.y);
    if (B.w != 0.f && q.z >= __fsub_rd(fminf(A.z, fminf(B.z, C.z)), zTolF) && q.z <= __fadd_ru(fmaxf(A.z, fmaxf(B.z, C.z)), zTolF) &&
        nearProjection(ax, ay, bx, by, cx, cy, epsSq)) {
        *onSurface = true;
        return 0;
    }
    const int u = edgeSign(bx, by, cx, cy);
    if (u == 0) return 0;
    const int v = edgeSign(cx, cy, ax, ay);
    if (v != u) return 0;
    const int w = edgeSign(ax, ay, bx, by);
    if (w != u) return 0;
    // inside the projected triangle, whose orientation (the sign of its normal's z) is u; the plane
    // meets the ray at z - qz = T / (U + V + W) with barycentric weights U, V, W
    const float U = det2(bx, cy, by, cx), V = det2(cx, ay, cy, ax), W = det2(ax, by, ay, bx);
    const float az = __fsub_rn(A.z, q.z), bz = __fsub_rn(B.z, q.z), cz = __fsub_rn(C.z, q.z);
    float T = fmaf(U, az, fmaf(V, bz, __fmul_rn(W, cz)));
    const float mag = fabsf(U * az) + fabsf(V * bz) + fabsf(W * cz);
    if (fabsf(T) <= 1e-6f * mag) {  // close to the plane: the height again in FP64 from exact weights
        const double Ud = double(bx) * double(cy) - double(by) * double(cx);
        const double Vd = double(cx) * double(ay) - double(cy) * double(ax);
        const double Wd = double(ax) * double(by) - double(ay) * double(bx);
        const double Td = Ud * (double(A.z) - double(q.z)) + Vd * (double(B.z) - double(q.z)) + Wd * (double(C.z) - double(q.z));
        T = Td > 0.0 ? 1.f : (Td < 0.0 ? -1.f : 0.f);
    }
    if (T == 0.f) {
        *onSurface = true;
        return 0;
    }
    const bool above = (T > 0.f) == (u > 0);
    if (above != up) return 0;
    return up ? u : -u;
}

// The exact winding number of a closed oriented surface at each lane's q with `need`: the signed
// number of crossings of the vertical ray from q (up when the warp's first lane lies in the upper
// half of the mesh's box, which shortens the rays), over the reference nodes' boxes (a ray meets a box
// when its (x, y) lies in the box's footprint and the box reaches past q along the ray).
// *onSurface: q lies on the surface (the caller evaluates the winding number there instead).
// skipSlot: a leaf slot whose triangle the lane's ray ignores (-1: none); *upOut: the rays' direction.
__device__ int rayWinding(const QueryTree& t, const float3& q, bool need, unsigned* status, bool* onSurface, int skipSlot = -1,
                          bool* upOut = nullptr) {
    const int lane = threadIdx.x & 31;
    int c = 0;
    const unsigned m0 = __ballot_sync(FULL, need);
    if (!m0 || t.nLeaves == 0) return 0;
    const bool up = __shfl_sync(FULL, q.z, __ffs(m0) - 1) >= 0.5f * (t.rootBox0.z + t.rootBox1.z);
    if (upOut) *upOut = up;
    const float epsSq = rayEpsSq(t), zTolF = __double2float_ru(rayZTol(t));
    WarpStack st;
    st.push(lane, 0, m0);
    bool overflow = false;
    while (st.sp > 0) {
        int node;
        unsigned m;
        st.pop(node, m);
        const float4 n0 = ld4(t.nodes + 2 * int64_t(node)), n1 = ld4(t.nodes + 2 * int64_t(node) + 1);
        const bool hit = ((m >> lane) & 1u) && q.x >= n0.x && q.x <= n0.w && q.y >= n0.y && q.y <= n1.x &&
                         (up ? n1.y >= q.z : n0.z <= q.z);
        const unsigned mh = __ballot_sync(FULL, hit);
        if (!mh) continue;
        const int l = __float_as_int(n1.z), r = __float_as_int(n1.w);
        if (r < 0) {  // a leaf: l is its face
            const int slot = t.faceSlot[l];
            const float4* tr = t.tri + 3 * int64_t(slot);
            const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
            if (hit && slot != skipSlot) c += rayCross(q, A, B, C, up, onSurface, epsSq, zTolF);
        } else {
            if (!st.push(lane, r, mh)) overflow = true;
            if (!st.push(lane, l, mh)) overflow = true;
            if (overflow) break;
        }
    }
    if (overflow && lane == 0) atomicOr(status, kStatusStackOverflow);
    return c;
}

// ------------------------------------------------------------------ sign columns (closed surfaces)
// One upward vertical ray per (x, y) column of a grid whose z axis is the world's (xf's third column
// (0, 0, +s)): every voxel of the column lies on that ray, so the exact winding number of a voxel is
// the signed number of the ray's crossings above it.  The crossings' heights come from the exact
// weights in FP64 (error below 1e-15 of the mesh's largest |z|); a voxel within 1e-12 of that of a
// crossing's height (on the surface, up to rounding), and every voxel of a column with more than
// kColumnCrossings crossings above its first voxel, gets the approximated winding number of the
// winding-number walk instead.
constexpr int kColumnCrossings = 24;

// The entry of triangle ABC in the list of the vertical column through q's (x, y): where the column
// crosses the triangle (the same exact, watertight projection test as rayCross), the tolerance
// interval of the crossing's height (FP64, from the exact weights) and its sign, the contribution to
// the winding number below it; where the column passes within sqrt(epsSq) of a vertical triangle
// (flagged in B.w: a voxel there may lie on the surface at any height of the triangle), an interval
// over the triangle's z range, plus zTol.
// The FP32 bounds compare with a voxel centre vz (a float) as the interval does: vz < lo <=> vz below
// it, vz > hi <=> vz above it (rounded outwards where widened).  false: no entry.
__device__ __forceinline__ bool columnEntry(const float3& q, const float4& A, const float4& B, const float4& C, double zTol,
                                            float zTolF, float epsSq, float* lo, float* hi, int* sign) {
    const float ax = __fsub_rn(A.x, q.x), ay = __fsub_rn(A.y, q.y), bx = __fsub_rn(B.x, q.x), by = __fsub_rn(B.y, q.y),
                cx = __fsub_rn(C.x, q.x), cy = __fsub_rn(C.y, q.y);
    const bool near = B.w != 0.f && nearProjection(ax, ay, bx, by, cx, cy, epsSq);
    const int u = edgeSign(bx, by, cx, cy);
    bool cross = u != 0 && edgeSign(cx, cy, ax, ay) == u && edgeSign(ax, ay, bx, by) == u;
    float l = FLT_MAX, h = -FLT_MAX;
    if (cross) {
        const double U = double(bx) * double(cy) - double(by) * double(cx);
        const double V = double(cx) * double(ay) - double(cy) * double(ax);
        const double W = double(ax) * double(by) - double(ay) * double(bx);
        const double det = U + V + W;
        if (det != 0.0) {
            const double z = (U * double(A.z) + V * double(B.z) + W * double(C.z)) / det;
            l = __double2float_ru(z - zTol);
            h = __double2float_rd(z + zTol);
        } else {
            cross = false;
        }
    }
    if (!cross && !near) return false;
    if (near) {
        l = fminf(l, __fsub_rd(fminf(A.z, fminf(B.z, C.z)), zTolF));
        h = fmaxf(h, __fadd_ru(fmaxf(A.z, fmaxf(B.z, C.z)), zTolF));
    }
    *lo = l;
    *hi = h;
    *sign = cross ? u : 0;
    return true;
}

// Crossing lists of the grid's columns, filled by columnRasterKernel: per column the number of
// crossings at or above the range's first voxel (may exceed kColumnSlots: the column then casts its
// own ray), bits 2k, 2k + 1 of signMask the sign of entry k (00: 0, 01: +1, 11: -1), and entry k's
// bounds {lo, hi} (columnEntry) at zz[k * ncols + column].  Index space of the columns:
// (fx, fy) = inv ((X, Y) - org); a column centre's FP32 (X, Y) lies within half of (ex, ey) of the
// exact one.
constexpr int kColumnSlots = 8;
struct ColumnLists {
    uint32_t* count;
    uint32_t* signMask;
    float2* zz;
    int64_t ncols;
    float inv[4], org[2];
    float ex, ey;
};

__device__ __forceinline__ void columnAdd(const ColumnLists& cl, const GridRange& g, const Xf& xf, double zTol, float zTolF,
                                          float epsSq, int ix, int iy, const float4& A, const float4& B, const float4& C) {
    const float3 q0 = xfPoint(xf, ix, iy, g.z0);
    float zl, zh;
    int sgn;
    if (!columnEntry(q0, A, B, C, zTol, zTolF, epsSq, &zl, &zh, &sgn)) return;
    if (q0.z > zh) return;  // below the range's first voxel
    const int64_t col = int64_t(iy) * g.nx + ix;
    const uint32_t k = atomicAdd(cl.count + col, 1u);
    if (k < uint32_t(kColumnSlots)) {
        cl.zz[size_t(k) * size_t(cl.ncols) + size_t(col)] = make_float2(zl, zh);
        if (sgn != 0) atomicOr(cl.signMask + col, (sgn > 0 ? 1u : 3u) << (2 * k));
    }
}

// One lane per triangle: the columns whose centre (x, y) may fall in the triangle's (x, y) bounds
// (the bounds widened by twice the centres' rounding, mapped to index space) are tested
// with columnEntry (the rays' exact crossing test, and the vertical-triangle rule), which adds each
// entry to its column's list.  A triangle
// over more than 16 candidate columns is taken by the whole warp, its lanes striding over them.
__global__ void __launch_bounds__(kThreads) columnRasterKernel(QueryTree t, GridRange g, Xf xf, ColumnLists cl) {
    const int lane = threadIdx.x & 31;
    const double zTol = rayZTol(t);
    const float zTolF = __double2float_ru(zTol), epsSq = rayEpsSq(t);
    const int64_t n = t.nLeaves;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i0 = int64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
        const int64_t i = i0 + lane;
        const bool active = i < n;
        float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A, C = A;
        int ix0 = 0, iy0 = 0, w = 0, h = 0;
        if (active) {
            const float4* tr = t.tri + 3 * i;
            A = ld4(tr);
            B = ld4(tr + 1);
            C = ld4(tr + 2);
            // the widened bounds relative to the grid's origin, mapped to index space in FP32 with a
            // margin of 1e-6 of the terms' magnitudes (about 17 ulps, several times the mapping's
            // rounding; FP64 issues far slower)
            const float x0 = __fsub_rn(__fsub_rn(fminf(A.x, fminf(B.x, C.x)), cl.ex), cl.org[0]);
            const float x1 = __fadd_rn(__fsub_rn(fmaxf(A.x, fmaxf(B.x, C.x)), cl.org[0]), cl.ex);
            const float y0 = __fsub_rn(__fsub_rn(fminf(A.y, fminf(B.y, C.y)), cl.ey), cl.org[1]);
            const float y1 = __fadd_rn(__fsub_rn(fmaxf(A.y, fmaxf(B.y, C.y)), cl.org[1]), cl.ey);
            float fx0 = FLT_MAX, fx1 = -FLT_MAX, fy0 = FLT_MAX, fy1 = -FLT_MAX;
            const bool finite = x0 <= x1 && y0 <= y1;  // (no candidates for non-finite bounds)
            for (int c = 0; c < 4 && finite; ++c) {
                const float X = (c & 1) ? x1 : x0, Y = (c & 2) ? y1 : y0;
                const float tx = fabsf(cl.inv[0] * X) + fabsf(cl.inv[1] * Y), ty = fabsf(cl.inv[2] * X) + fabsf(cl.inv[3] * Y);
                const float fx = fmaf(cl.inv[0], X, cl.inv[1] * Y), fy = fmaf(cl.inv[2], X, cl.inv[3] * Y);
                fx0 = fminf(fx0, fx - 1e-6f * tx);
                fx1 = fmaxf(fx1, fx + 1e-6f * tx);
                fy0 = fminf(fy0, fy - 1e-6f * ty);
                fy1 = fmaxf(fy1, fy + 1e-6f * ty);
            }
            // the candidates: ceil(f0) .. floor(f1), clamped to the grid (compared in FP32 before any
            // conversion, so bounds beyond int range convert nothing)
            const float cx0 = fmaxf(0.f, ceilf(fx0)), cx1 = fminf(float(g.nx - 1), floorf(fx1));
            const float cy0 = fmaxf(0.f, ceilf(fy0)), cy1 = fminf(float(g.ny - 1), floorf(fy1));
            if (finite && cx0 <= cx1 && cy0 <= cy1) {
                ix0 = int(cx0);
                iy0 = int(cy0);
                w = int(cx1) - ix0 + 1;
                h = int(cy1) - iy0 + 1;
            }
        }
        const int64_t nc = int64_t(w) * h;
        if (nc <= 16) {
            for (int c = 0; c < int(nc); ++c) columnAdd(cl, g, xf, zTol, zTolF, epsSq, ix0 + c % w, iy0 + c / w, A, B, C);
        }
        unsigned big = __ballot_sync(FULL, nc > 16);
        while (big) {
            const int b = __ffs(big) - 1;
            big &= big - 1;
            // the whole records, flags included (B.w: a vertical triangle)
            const float4 Ab = make_float4(__shfl_sync(FULL, A.x, b), __shfl_sync(FULL, A.y, b), __shfl_sync(FULL, A.z, b),
                                          __shfl_sync(FULL, A.w, b));
            const float4 Bb = make_float4(__shfl_sync(FULL, B.x, b), __shfl_sync(FULL, B.y, b), __shfl_sync(FULL, B.z, b),
                                          __shfl_sync(FULL, B.w, b));
            const float4 Cb = make_float4(__shfl_sync(FULL, C.x, b), __shfl_sync(FULL, C.y, b), __shfl_sync(FULL, C.z, b),
                                          __shfl_sync(FULL, C.w, b));
            const int bx0 = __shfl_sync(FULL, ix0, b), by0 = __shfl_sync(FULL, iy0, b), bw = __shfl_sync(FULL, w, b);
            const int64_t bn = int64_t(bw) * __shfl_sync(FULL, h, b);
            for (int64_t c = lane; c < bn; c += 32)
                columnAdd(cl, g, xf, zTol, zTolF, epsSq, bx0 + int(c % bw), by0 + int(c / bw), Ab, Bb, Cb);
        }
    }
}

// For the grid columns of the launch (32 consecutive x per warp, in segments of kColumnSeg layers;
// the crossings from the columns' lists, or a column's own ray where its list overflowed or there are
// no lists): inside = (winding number of the voxel > threshold), written as bits (one
// word per 32 voxels along x, layout (z - zOut, y, x / 32)) or applied to `values` (negated where
// inside; value index (z - zOut) nx ny + y nx + x).  The range [z0, z1) of dims is covered.
constexpr int kColumnSeg = 128;

// Inside bits (bit k: the voxel at zc + k) of the voxels of a column chunk marked in `amb`, from their
// approximated winding numbers.  Out of line, as columnRay: few voxels take it.
template <bool PRECISE>
__device__ __noinline__ uint32_t columnWalks(const QueryTree& t, const Xf& xf, int xc, int y, int zc, int kn, uint32_t amb,
                                             float betaSq, float threshold, unsigned* status) {
    uint32_t in = 0;
    for (int k = 0; k < kn; ++k) {
        const bool need = (amb >> k) & 1u;
        if (!__any_sync(FULL, need)) continue;
        const float wf = fwnPacket<PRECISE>(t, xfPoint(xf, xc, y, zc + k), need, betaSq, -1, status);
        if (need && wf > threshold) in |= 1u << k;
    }
    return in;
}

// The entries of the columns of the lanes with `ray` from their own vertical ray: a packet walk over
// the reference nodes (a node when the lane's (x, y) lies in its box's footprint and the box reaches
// q0's height) adding each triangle's columnEntry to the lane's list, by lo; past kColumnCrossings
// entries, or when the stack overflows (the whole warp), *overflow is set.  Out of line: only
// columns whose list overflowed, or launches without lists, take it, and its registers stay out of
// the sweep.
__device__ __noinline__ void columnRay(const QueryTree& t, float3 q0, bool ray, double zTol, float zTolF, float epsSq, float* lo,
                                       float* hi, int* sg, int* nOut, bool* overflowOut, unsigned* status) {
    const int lane = threadIdx.x & 31;
    int n = *nOut;
    bool overflow = *overflowOut;
    WarpStack st;
    st.push(lane, 0, __ballot_sync(FULL, ray));
    bool stackFull = false;
    while (st.sp > 0 && t.nLeaves > 0) {
        int node;
        unsigned m;
        st.pop(node, m);
        const float4 n0 = ld4(t.nodes + 2 * int64_t(node)), n1 = ld4(t.nodes + 2 * int64_t(node) + 1);
        const bool hit = ((m >> lane) & 1u) && q0.x >= n0.x && q0.x <= n0.w && q0.y >= n0.y && q0.y <= n1.x && n1.y >= q0.z;
        const unsigned mh = __ballot_sync(FULL, hit);
        if (!mh) continue;
        const int l = __float_as_int(n1.z), r = __float_as_int(n1.w);
        if (r < 0) {
            const float4* tr = t.tri + 3 * int64_t(t.faceSlot[l]);
            const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
            float zl, zh;
            int sgn;
            if (hit && columnEntry(q0, A, B, C, zTol, zTolF, epsSq, &zl, &zh, &sgn) && !(q0.z > zh)) {
                if (n < kColumnCrossings) {
                    int k = n++;
                    while (k > 0 && lo[k - 1] > zl) {
                        lo[k] = lo[k - 1];
                        hi[k] = hi[k - 1];
                        sg[k] = sg[k - 1];
                        --k;
                    }
                    lo[k] = zl;
                    hi[k] = zh;
                    sg[k] = sgn;
                } else {
                    overflow = true;
                }
            }
        } else if (!st.push(lane, r, mh) || !st.push(lane, l, mh)) {
            stackFull = true;
            break;
        }
    }
    if (stackFull) {
        overflow = true;  // every lane of the warp falls back
        if (lane == 0) atomicOr(status, kStatusStackOverflow);
    }
    *nOut = n;
    *overflowOut = overflow;
}

template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, 4) signColumnsKernel(QueryTree t, GridRange g, Xf xf, float threshold, float beta,
                                                          uint32_t* __restrict__ bits, float* __restrict__ values,
                                                          ColumnLists cl, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const float betaSq = __fmul_rn(beta, beta);
    const int wordsX = (g.nx + 31) >> 5;
    const int segs = (g.z1 - g.z0 + kColumnSeg - 1) / kColumnSeg;
    const uint64_t items = uint64_t(wordsX) * uint64_t(g.ny) * uint64_t(segs);
    const size_t sxy = size_t(g.nx) * g.ny;
    const double zTol = rayZTol(t);
    const float zTolF = __double2float_ru(zTol), epsSq = rayEpsSq(t);
    // per entry (ascending lo; columnEntry): the FP32 bounds of its interval, so that for a voxel
    // centre vz (a float) vz < lo <=> vz below the interval and vz > hi <=> vz above it: the sweep
    // compares in FP32 (FP64 issues at a small fraction of the FP32 rate)
    float lo[kColumnCrossings], hi[kColumnCrossings];
    int sg[kColumnCrossings];
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= items) break;
        const int wx = int(item % unsigned(wordsX));
        const unsigned rest = item / unsigned(wordsX);
        const int y = int(rest % unsigned(g.ny));
        const int zs0 = g.z0 + int(rest / unsigned(g.ny)) * kColumnSeg, zs1 = min(g.z1, zs0 + kColumnSeg);
        const int x = wx * 32 + lane;
        const bool active = x < g.nx;
        const int xc = active ? x : 0;
        const float3 q0 = xfPoint(xf, xc, y, zs0);
        // the column's crossings from its list, or, without lists or when the list overflowed, from
        // the ray: a packet walk over the reference nodes collecting the crossings above q0; by height
        int n = 0;
        bool overflow = false;
        bool ray = active && !cl.count;
        if (cl.count && active) {
            const int64_t col = int64_t(y) * g.nx + x;
            const uint32_t c = __ldg(cl.count + col);
            if (c <= uint32_t(kColumnSlots)) {
                const uint32_t mask = __ldg(cl.signMask + col);
                for (uint32_t e = 0; e < c; ++e) {
                    const float2 zz = __ldg(cl.zz + size_t(e) * size_t(cl.ncols) + size_t(col));
                    int k = n++;
                    while (k > 0 && lo[k - 1] > zz.x) {
                        lo[k] = lo[k - 1];
                        hi[k] = hi[k - 1];
                        sg[k] = sg[k - 1];
                        --k;
                    }
                    lo[k] = zz.x;
                    hi[k] = zz.y;
                    const uint32_t m2 = (mask >> (2 * e)) & 3u;
                    sg[k] = m2 == 1u ? 1 : (m2 == 3u ? -1 : 0);
                }
            } else {
                ray = true;
            }
        }
        if (__any_sync(FULL, ray)) columnRay(t, q0, ray, zTol, zTolF, epsSq, lo, hi, sg, &n, &overflow, scratch + 1);
        // the sweep up the segment, 32 layers at a time: w = signed crossings above the voxel
        int w = 0, p = 0;
        for (int k = 0; k < n; ++k) w += sg[k];
        for (int zc = zs0; zc < zs1; zc += 32) {
            const int kn = min(32, zs1 - zc);
            uint32_t in = 0, amb = 0;  // bit k: the voxel at zc + k
            for (int k = 0; k < kn; ++k) {
                const float vz = xfPoint(xf, xc, y, zc + k).z;
                // entries passed (below the voxel) leave w; the walk stops at the first entry reaching
                // up to vz, and every entry after it starts above lo[p] (ascending lo): so the voxel
                // lies in an interval iff vz >= lo[p], and otherwise every entry left is above it
                while (p < n && vz > hi[p]) {
                    w -= sg[p];
                    ++p;
                }
                if (overflow || (p < n && vz >= lo[p]))  // on the surface, up to rounding: the walk decides
                    amb |= 1u << k;
                else if (float(w) > threshold)
                    in |= 1u << k;
            }
            if (!active) amb = in = 0;
            // on the surface (up to rounding): the winding-number walk
            if (__any_sync(FULL, amb != 0)) in |= columnWalks<PRECISE>(t, xf, xc, y, zc, kn, amb, betaSq, threshold, scratch + 1);
            if (values) {
                float* vp = values + size_t(zc - g.zOut) * sxy + size_t(y) * g.nx + xc;
#pragma unroll 8
                for (int k = 0; k < kn; ++k)
                    if ((in >> k) & 1u) vp[size_t(k) * sxy] = -vp[size_t(k) * sxy];
            } else {
                uint32_t mine = 0;  // lane k stores layer zc + k's word
                for (int k = 0; k < kn; ++k) {
                    const uint32_t word = __ballot_sync(FULL, (in >> k) & 1u);
                    if (lane == k) mine = word;
                }
                if (lane < kn) bits[(size_t(zc + lane - g.zOut) * g.ny + y) * wordsX + wx] = mine;
            }
        }
    }
}

// True when a voxel at q may take the sign of the voxel at qb, whose squared distance to the surface
// is belowSq (> 0, from a search that ran to the end): qb is farther from the surface than from q, so
// the segment between them meets no surface.  The margin covers the FP32 rounding of both centres and
// of the distance, relative to the coordinates' magnitude.  qb must be computed exactly as that
// voxel's centre was (the same xfPoint call).
__device__ __forceinline__ bool emptyBallCovers(const float3& q, const float3& qb, float belowSq) {
    const float dx = q.x - qb.x, dy = q.y - qb.y, dz = q.z - qb.z;
    const float step = sqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
    const float db = sqrtf(belowSq);
    const float mag = fmaxf(fabsf(q.x), fmaxf(fabsf(q.y), fabsf(q.z)));
    return db > fmaf(step, 1.0001f, 2e-6f * fmaf(3.f, mag, db));
}

// Sign reuse for one tile of TX x TY x TZ voxels (lane = lx + TX (ly + TY lz)) after its closest-point
// searches.  below: the state of the voxel that precedes this lane's voxel (the previous tile's top
// layer for the bottom layer, the lane's own voxel of the previous tile for the others): its squared
// distance with its side in the sign bit, NaN when unknown; zb: that voxel's layer.  A lane above the
// bottom layer may also take the sign of the voxel one layer below it in this tile, once that one's
// sign is settled by reuse.  Returns whether the lane's sign is settled; *inside receives it.
template <int TX, int TY, int TZ>
__device__ __forceinline__ bool reuseSign(const Xf& xf, int x, int y, int z, int zb, int lz, const float3& q, float below,
                                          bool complete, float dsq, bool* inside) {
    bool reuse = fabsf(below) > 0.f && emptyBallCovers(q, xfPoint(xf, x, y, zb), fabsf(below));
    bool in = signbit(below);
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int l = 1; l < TZ; ++l) {
        const float e = __shfl_sync(FULL, (reuse && complete) ? (in ? -dsq : dsq) : __int_as_float(0x7fc00000),
                                    lane >= TX * TY ? lane - TX * TY : lane);
        if (lz == l && !reuse && fabsf(e) > 0.f && emptyBallCovers(q, xfPoint(xf, x, y, z - 1), fabsf(e))) {
            reuse = true;
            in = signbit(e);
        }
    }
    *inside = in;
    return reuse;
}

// A warp takes a column of tiles along z and walks it upwards.  Each lane starts its closest-point
// search from the triangle that was closest to a voxel just below its own: the bottom layer of a
// tile from the voxel one layer below (the previous tile's top layer), the top layer from its own
// voxel of the previous tile, two layers below.  That triangle's distance is an upper bound the
// search would reach anyway, so the minimum is unchanged, but it prunes from the first step (a third
// fewer node visits with an exact bound, in a CPU model of the walk).  On a closed surface the same
// voxel below also lends its sign (signReuseAllowed) when its distance exceeds the step between the
// two voxel centres, and the lane skips its winding-number walk.
template <bool PRECISE, bool DIST, bool BITS = false>
__global__ void __launch_bounds__(kThreads, DIST ? kDistBlocks : 4) gridKernel(QueryTree t, GridRange g, TileGrid tg, Xf xf, DistOpts o,
                                                       float* __restrict__ out, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % kTX, ly = (lane / kTX) % kTY, lz = lane / (kTX * kTY);
    const float betaSq = __fmul_rn(o.beta, o.beta);
    const size_t sxy = size_t(g.nx) * g.ny;
    const bool reuseOk = DIST && !BITS && signReuseAllowed(t, o);
    const int wordsX = (g.nx + 31) >> 5;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= tg.numItems) break;
        int x0, y0, zBase, nSeg;
        if (tg.runs) {
            const int4 r = tg.runs[item / kBrickCols];
            const int col = int(item % kBrickCols);
            x0 = r.x * 8 + (col % kBrickColsX) * kTX;
            y0 = r.y * 8 + (col / kBrickColsX) * kTY;
            zBase = g.z0 + r.z * 8;
            nSeg = kBrickSeg * r.w;
        } else {
            const int tx = int(item % unsigned(tg.tilesX));
            const unsigned rest = item / unsigned(tg.tilesX);
            const int ty = int(rest % unsigned(tg.tilesY));
            const int sz = int(rest / unsigned(tg.tilesY));
            x0 = tx * kTX;
            y0 = ty * kTY;
            zBase = g.z0 + sz * tg.segLen * kTZ;
            nSeg = min(tg.segLen, tg.tilesZ - sz * tg.segLen);
        }
        const int x = x0 + lx, y = y0 + ly;
        int seed = -1;  // leaf slot closest to the voxel below
        // that voxel's squared distance with its side in the sign bit (negative inside), NaN when
        // its sign is unknown
        float below = __int_as_float(0x7fc00000);
        const uint32_t colsPerSlab = uint32_t(tg.tilesX) * uint32_t(tg.tilesY);
        if (DIST && tg.colState && !tg.runs && item >= colsPerSlab) {
            // the column below ended (its state was written) or not yet (0xff bytes: start cold); the
            // voxel below both layers of the first tile is that column's top-layer voxel
            const float* cs = tg.colState + size_t(item - colsPerSlab) * (2 * kLayer);
            if (!BITS) below = __ldcg(cs + lane % kLayer);
            seed = __float_as_int(__ldcg(cs + kLayer + lane % kLayer));
        }
        for (int j = 0; j < nSeg; ++j) {
            const int z = zBase + j * kTZ + lz;
            const bool active = x < g.nx && y < g.ny && z < g.z1;
            const float3 q = xfPoint(xf, x, y, z);
            float res;
            if (DIST) {
                float up = o.maxDistSq;
                if (active && seed >= 0) {
                    const float4* tr = t.tri + 3 * int64_t(seed);
                    const float ds = triDistSq<PRECISE>(q, ld4(tr), ld4(tr + 1), ld4(tr + 2));
                    if (ds < up) up = ds;
                }
                int best = active ? seed : -1;
                const float dsq = cpPacket<PRECISE, true>(t, q, active, up, o.minDistSq, scratch + 1, &best);
                const bool valid = !(o.nullOutsideMinMax && (dsq < o.minDistSq || dsq >= o.maxDistSq));
                const bool complete = active && valid && dsq >= o.minDistSq;
                bool inside;
                if (BITS) {  // the column rays' signs
                    const uint32_t word = active ? __ldg(tg.signBits + (size_t(z - g.zOut) * g.ny + y) * wordsX + (x >> 5)) : 0u;
                    inside = (word >> (x & 31)) & 1u;
                } else {
                    bool reIn = false;
                    const bool reuse = reuseOk && reuseSign<kTX, kTY, kTZ>(xf, x, y, z, z - (lz == 0 ? 1 : kTZ), lz, q, below,
                                                                          complete, dsq, &reIn);
                    // closed surface: the exact winding number from ray crossings, but the approximated
                    // one (the reference's decision) for a voxel on the surface; otherwise the latter
                    bool onSurface = false;
                    const int cw = reuseOk ? rayWinding(t, q, active && valid && !reuse, scratch + 1, &onSurface) : 0;
                    const bool fwn = reuseOk ? onSurface : (active && valid);
                    const float w = fwnPacket<PRECISE>(t, q, fwn, betaSq, -1, scratch + 1);
                    inside = reuse ? reIn : (fwn ? w > o.threshold : float(cw) > o.threshold);
                }
                const float d = __fsqrt_rn(dsq);
                res = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
                // next tile: the bottom layer's lanes take the voxel one layer below them (this tile's
                // top layer), the others their own voxel two layers below.  A distance counts only when
                // the search ran to the end (not cut short below minDistSq): no surface is closer then.
                const int src = lane + (kTZ - 1) * kTX * kTY * (lz == 0);
                seed = __shfl_sync(FULL, best, src);
                if (!BITS) below = __shfl_sync(FULL, complete ? (inside ? -dsq : dsq) : __int_as_float(0x7fc00000), src);
                if (tg.colState && !tg.runs && j == nSeg - 1 && lz == kTZ - 1) {
                    // the column's last tile: the top layer's lanes hold their own voxels' state and
                    // pass on the distances and the seeds at this work item's words (the item
                    // recomputed from the column's position, so no register holds it through the walk)
                    const uint32_t sz = uint32_t(zBase - g.z0) / uint32_t(tg.segLen * kTZ);
                    const uint32_t it = uint32_t(x0) / kTX + uint32_t(tg.tilesX) * (uint32_t(y0) / kTY + uint32_t(tg.tilesY) * sz);
                    float* cs = tg.colState + size_t(it) * (2 * kLayer) + (lane - (kTZ - 1) * kLayer);
                    cs[0] = below;
                    cs[kLayer] = __int_as_float(seed);
                }
            } else {
                res = fwnPacket<PRECISE>(t, q, active, betaSq, -1, scratch + 1);
            }
            if (active) out[size_t(z - g.zOut) * sxy + size_t(y) * g.nx + x] = res;
        }
    }
}

// Signed distances with the column pass's sign bits and no lower distance bound (minDistSq = 0): a
// warp walks its column two tiles at a time, each lane taking its voxel of the lower tile and the one
// two layers above it (a 4x4x4 block of voxels) through one shared packet walk (cpPacket2), so each
// record read and stack step serves 64 voxels.  Both start from the triangle closest to the voxel
// below the lower tile (as gridKernel's seeds); results are the exact minima, as gridKernel's.  In
// precise mode the walk runs in FP32 and the voxels that came within a triangle's near-plane level
// are listed for fixPairKernel, which walks them again with the precise distances.
template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, kPairBlocks) gridPairKernel(QueryTree t, GridRange g, TileGrid tg, Xf xf, DistOpts o,
                                                                        float* __restrict__ out, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % kTX, ly = (lane / kTX) % kTY, lz = lane / (kTX * kTY);
    const size_t sxy = size_t(g.nx) * g.ny;
    const int wordsX = (g.nx + 31) >> 5;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= tg.numItems) break;
        int x0, y0, zBase, nSeg;
        if (tg.runs) {
            const int4 r = tg.runs[item / kBrickCols];
            const int col = int(item % kBrickCols);
            x0 = r.x * 8 + (col % kBrickColsX) * kTX;
            y0 = r.y * 8 + (col / kBrickColsX) * kTY;
            zBase = g.z0 + r.z * 8;
            nSeg = kBrickSeg * r.w;
        } else {
            const int tx = int(item % unsigned(tg.tilesX));
            const unsigned rest = item / unsigned(tg.tilesX);
            const int ty = int(rest % unsigned(tg.tilesY));
            const int sz = int(rest / unsigned(tg.tilesY));
            x0 = tx * kTX;
            y0 = ty * kTY;
            zBase = g.z0 + sz * tg.segLen * kTZ;
            nSeg = min(tg.segLen, tg.tilesZ - sz * tg.segLen);
        }
        const int x = x0 + lx, y = y0 + ly;
        int seed = -1;
        const uint32_t colsPerSlab = uint32_t(tg.tilesX) * uint32_t(tg.tilesY);
        if (tg.colState && !tg.runs && item >= colsPerSlab)
            seed = __float_as_int(__ldcg(tg.colState + size_t(item - colsPerSlab) * (2 * kLayer) + kLayer + lane % kLayer));
        for (int j = 0; j < nSeg; j += 2) {
            const bool hasB = j + 1 < nSeg;
            const int za = zBase + j * kTZ + lz, zb = za + kTZ;
            const bool inXY = x < g.nx && y < g.ny;
            const bool activeA = inXY && za < g.z1, activeB = inXY && hasB && zb < g.z1;
            const float3 qa = xfPoint(xf, x, y, za), qb = xfPoint(xf, x, y, zb);
            float ra = o.maxDistSq, rb = o.maxDistSq;
            int ba = -1, bb = -1;
            if (PRECISE) {
                if (lane == 0) sPairFix[threadIdx.x >> 5][0] = sPairFix[threadIdx.x >> 5][1] = 0u;
                __syncwarp();
            }
            if (seed >= 0 && (activeA || activeB)) {
                bool da = false, db = false;
                leafDist2<PRECISE>(t, seed, qa, qb, activeA, activeB, ra, rb, ba, bb, da, db);
            }
            cpPacket2<PRECISE>(t, qa, qb, activeA, activeB, ra, rb, ba, bb, scratch + 1);
            if (PRECISE) {
                __syncwarp();
                const unsigned ma = sPairFix[threadIdx.x >> 5][0], mb = sPairFix[threadIdx.x >> 5][1];
                if ((ma | mb) && lane == 0) {  // re-walked with the precise distances by fixPairKernel
                    const uint32_t k = atomicAdd(&tg.fixList[0].x, 1u);
                    if (k < tg.fixCap) tg.fixList[1 + k] = make_uint4(item, uint32_t(j), ma, mb);
                }
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const bool active = h ? activeB : activeA;
                const int z = h ? zb : za;
                const float dsq = h ? rb : ra;
                const bool valid = !(o.nullOutsideMinMax && dsq >= o.maxDistSq);
                const uint32_t word = active ? __ldg(tg.signBits + (size_t(z - g.zOut) * g.ny + y) * wordsX + (x >> 5)) : 0u;
                const bool inside = (word >> (x & 31)) & 1u;
                const float d = __fsqrt_rn(dsq);
                if (active) out[size_t(z - g.zOut) * sxy + size_t(y) * g.nx + x] = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
            }
            // next pair: the bottom layer's lanes continue from the voxel one layer below them, the
            // others from their own last voxel (as gridKernel)
            const int src = lane + (kTZ - 1) * kTX * kTY * (lz == 0);
            seed = __shfl_sync(FULL, hasB ? bb : ba, src);
            if (tg.colState && !tg.runs && j + 2 >= nSeg && lz == kTZ - 1) {
                // the column's last tile: its top layer passes its closest triangles to the column above
                const uint32_t sz = uint32_t(zBase - g.z0) / uint32_t(tg.segLen * kTZ);
                const uint32_t it = uint32_t(x0) / kTX + uint32_t(tg.tilesX) * (uint32_t(y0) / kTY + uint32_t(tg.tilesY) * sz);
                float* cs = tg.colState + size_t(it) * (2 * kLayer) + (lane - (kTZ - 1) * kLayer);
                cs[0] = __int_as_float(0x7fc00000);
                cs[kLayer] = __int_as_float(seed);
            }
        }
    }
}

// Winding numbers of a grid two tiles at a time (fwnPacket2): each lane takes its voxel of the lower
// tile and the one kTZ layers above; the same values as gridKernel<PRECISE, false>, bit for bit.
// 4 blocks per SM (64 registers): at 512^3 on 1.31 M triangles 19.7 ms, against 20.7 ms at 3 and
// 29.6 ms at 5 (spills).
template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, 4) gridFwnPairKernel(QueryTree t, GridRange g, TileGrid tg, Xf xf, float beta,
                                                                 float* __restrict__ out, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % kTX, ly = (lane / kTX) % kTY, lz = lane / (kTX * kTY);
    const float betaSq = __fmul_rn(beta, beta);
    const size_t sxy = size_t(g.nx) * g.ny;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= tg.numItems) break;
        const int tx = int(item % unsigned(tg.tilesX));
        const unsigned rest = item / unsigned(tg.tilesX);
        const int ty = int(rest % unsigned(tg.tilesY));
        const int sz = int(rest / unsigned(tg.tilesY));
        const int x = tx * kTX + lx, y = ty * kTY + ly;
        const int zBase = g.z0 + sz * tg.segLen * kTZ;
        const int nSeg = min(tg.segLen, tg.tilesZ - sz * tg.segLen);
        for (int j = 0; j < nSeg; j += 2) {
            const int za = zBase + j * kTZ + lz, zb = za + kTZ;
            const bool inXY = x < g.nx && y < g.ny;
            const bool activeA = inXY && za < g.z1, activeB = inXY && j + 1 < nSeg && zb < g.z1;
            float wa, wb;
            fwnPacket2<PRECISE>(t, xfPoint(xf, x, y, za), xfPoint(xf, x, y, zb), activeA, activeB, betaSq, scratch + 1, &wa, &wb);
            if (activeA) out[size_t(za - g.zOut) * sxy + size_t(y) * g.nx + x] = wa;
            if (activeB) out[size_t(zb - g.zOut) * sxy + size_t(y) * g.nx + x] = wb;
        }
    }
}

// Winding numbers of spatially ordered points, two tiles of 32 per work item (fwnPacket2): lane i takes
// the i-th point of each tile; the same values as vectorKernel<PRECISE, false>, bit for bit.
template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, 4) vectorFwnPairKernel(QueryTree t, const float* __restrict__ pts, int64_t n,
                                                                   float beta, float* __restrict__ out, unsigned* scratch,
                                                                   const int32_t* __restrict__ order) {
    const int lane = threadIdx.x & 31;
    const float betaSq = __fmul_rn(beta, beta);
    const uint64_t numPairs = (uint64_t(n) + 63) / 64;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (item >= numPairs) break;
        const int64_t ra = int64_t(item) * 64 + lane, rb = ra + 32;  // ranks in processing order
        const bool activeA = ra < n, activeB = rb < n;
        const int64_t ia = activeA ? int64_t(order[ra]) : 0, ib = activeB ? int64_t(order[rb]) : 0;
        float3 qa = make_float3(0.f, 0.f, 0.f), qb = qa;
        if (activeA) qa = make_float3(pts[3 * ia], pts[3 * ia + 1], pts[3 * ia + 2]);
        if (activeB) qb = make_float3(pts[3 * ib], pts[3 * ib + 1], pts[3 * ib + 2]);
        float wa, wb;
        fwnPacket2<PRECISE>(t, qa, qb, activeA, activeB, betaSq, scratch + 1, &wa, &wb);
        if (activeA) out[ia] = wa;
        if (activeB) out[ib] = wb;
    }
}

// The listed pair steps of a precise gridPairKernel launch: each flagged voxel's closest distance by
// the precise walk (cpPacket, from maxDistSq), written with its sign bit.  Voxels never listed kept
// FP32 distances no triangle came near the FP64 re-evaluation for: the precise walk's own.  A list
// that overflowed (more flagged steps than a launch has) cannot happen: one entry per step at most.
__global__ void __launch_bounds__(kThreads) fixPairKernel(QueryTree t, GridRange g, TileGrid tg, Xf xf, DistOpts o,
                                                          float* __restrict__ out, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % kTX, ly = (lane / kTX) % kTY, lz = lane / (kTX * kTY);
    const size_t sxy = size_t(g.nx) * g.ny;
    const int wordsX = (g.nx + 31) >> 5;
    const uint32_t n = min(__ldcg(&tg.fixList[0].x), tg.fixCap);
    for (;;) {
        const unsigned e = nextTicket(scratch, lane);
        if (e >= n) break;
        const uint4 f = tg.fixList[1 + e];
        const unsigned item = f.x;
        int x0, y0, zBase;
        if (tg.runs) {
            const int4 r = tg.runs[item / kBrickCols];
            const int col = int(item % kBrickCols);
            x0 = r.x * 8 + (col % kBrickColsX) * kTX;
            y0 = r.y * 8 + (col / kBrickColsX) * kTY;
            zBase = g.z0 + r.z * 8;
        } else {
            const unsigned rest = item / unsigned(tg.tilesX);
            x0 = int(item % unsigned(tg.tilesX)) * kTX;
            y0 = int(rest % unsigned(tg.tilesY)) * kTY;
            zBase = g.z0 + int(rest / unsigned(tg.tilesY)) * tg.segLen * kTZ;
        }
        const int x = x0 + lx, y = y0 + ly;
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            const bool need = ((h ? f.w : f.z) >> lane) & 1u;
            if (!__any_sync(FULL, need)) continue;
            const int z = zBase + (int(f.y) + h) * kTZ + lz;
            const float3 q = xfPoint(xf, x, y, z);
            const float dsq = cpPacket<true>(t, q, need, o.maxDistSq, 0.f, scratch + 1);
            if (need) {
                const bool valid = !(o.nullOutsideMinMax && dsq >= o.maxDistSq);
                const uint32_t word = __ldg(tg.signBits + (size_t(z - g.zOut) * g.ny + y) * wordsX + (x >> 5));
                const float d = __fsqrt_rn(dsq);
                out[size_t(z - g.zOut) * sxy + size_t(y) * g.nx + x] =
                    valid ? (((word >> (x & 31)) & 1u) ? -d : d) : __int_as_float(0x7fc00000);
            }
        }
    }
}

// A warp takes `chunk` consecutive tiles of 32 points; with Morton-ordered points a lane's point in
// one tile is near its point in the previous one, so (as in gridKernel) each lane starts its
// closest-point search from the triangle closest to its previous point.
template <bool PRECISE, bool DIST>
__global__ void __launch_bounds__(kThreads, DIST ? kDistBlocks : 4) vectorKernel(QueryTree t, const float* __restrict__ pts, int64_t n, DistOpts o,
                                                         int32_t skipFace, float* __restrict__ out, unsigned* scratch,
                                                         const int32_t* __restrict__ order, int chunk) {
    const int lane = threadIdx.x & 31;
    const float betaSq = __fmul_rn(o.beta, o.beta);
    const int skipSlot = (skipFace >= 0 && skipFace < t.nFaces) ? t.faceSlot[skipFace] : -1;
    const uint64_t numTiles = (uint64_t(n) + 31) / 32;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (uint64_t(item) * chunk >= numTiles) break;
        int seed = -1;
        for (int j = 0; j < chunk; ++j) {
            const uint64_t tile = uint64_t(item) * chunk + j;
            if (tile >= numTiles) break;
            const int64_t r = int64_t(tile) * 32 + lane;  // rank in processing order
            const bool active = r < n;
            const int64_t i = (order && active) ? int64_t(order[r]) : r;
            float3 q = make_float3(0.f, 0.f, 0.f);
            if (active) q = make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
            float res;
            if (DIST) {
                float up = o.maxDistSq;
                if (active && seed >= 0) {
                    const float4* tr = t.tri + 3 * int64_t(seed);
                    const float ds = triDistSq<PRECISE>(q, ld4(tr), ld4(tr + 1), ld4(tr + 2));
                    if (ds < up) up = ds;
                }
                int best = active ? seed : -1;
                const float dsq = cpPacket<PRECISE, true>(t, q, active, up, o.minDistSq, scratch + 1, &best);
                seed = best;
                const bool valid = !(o.nullOutsideMinMax && (dsq < o.minDistSq || dsq >= o.maxDistSq));
                // closed surfaces: the exact winding number from ray crossings (gridKernel)
                bool onSurface = false;
                const bool rays = signReuseAllowed(t, o);
                const int cw = rays ? rayWinding(t, q, active && valid, scratch + 1, &onSurface) : 0;
                const bool fwn = rays ? onSurface : (active && valid);
                const float w = fwnPacket<PRECISE>(t, q, fwn, betaSq, -1, scratch + 1);
                const bool inside = fwn ? w > o.threshold : float(cw) > o.threshold;
                const float d = __fsqrt_rn(dsq);
                res = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
            } else {
                res = fwnPacket<PRECISE>(t, q, active, betaSq, skipSlot, scratch + 1);
            }
            if (active) out[i] = res;
        }
    }
}

// Closest point with barycentric coordinates, FP64 (MRMesh/MRClosestPointInTriangle.h:28-91, in
// double as MRMesh/MRMeshProject.cpp:66-72 calls it): proj = (1 - ba - bb) a + ba b + bb c.
__device__ __noinline__ void closestPointBaryFp64(const float3 p, const float4 A, const float4 B, const float4 C, float3* proj,
                                                  float* ba, float* bb) {
    using V = V3T<double>;
    const V pd{p.x, p.y, p.z}, a{A.x, A.y, A.z}, b{B.x, B.y, B.z}, c{C.x, C.y, C.z};
    const V ab = vsub(b, a), ac = vsub(c, a), ap = vsub(pd, a);
    V r;
    double u = 0, w = 0;
    const double d1 = vdot(ab, ap), d2 = vdot(ac, ap);
    const V bp = vsub(pd, b);
    const double d3 = vdot(ab, bp), d4 = vdot(ac, bp);
    const V cp = vsub(pd, c);
    const double d5 = vdot(ab, cp), d6 = vdot(ac, cp);
    const double vc = d1 * d4 - d3 * d2, vb = d5 * d2 - d1 * d6, va = d3 * d6 - d5 * d4;
    if (d1 <= 0 && d2 <= 0) {
        r = a;
    } else if (d3 >= 0 && d4 <= d3) {
        r = b;
        u = 1;
    } else if (d6 >= 0 && d5 <= d6) {
        r = c;
        w = 1;
    } else if (vc <= 0 && d1 >= 0 && d3 <= 0) {
        u = d1 / (d1 - d3);
        r = vmad(a, u, ab);
    } else if (vb <= 0 && d6 <= 0 && d2 >= 0) {
        w = d2 / (d2 - d6);
        r = vmad(a, w, ac);
    } else if (va <= 0) {
        if (d4 < d3) {
            r = b;
            u = 1;
        } else if (d5 < d6) {
            r = c;
            w = 1;
        } else {
            const double v = (d4 - d3) / ((d4 - d3) + (d5 - d6));
            r = vmad(b, v, vsub(c, b));
            u = 1 - v;
            w = v;
        }
    } else {
        const double denom = 1 / (va + vb + vc);
        u = vb * denom;
        w = vc * denom;
        r = vmad(vmad(a, u, ab), w, ac);
    }
    *proj = make_float3(float(r.x), float(r.y), float(r.z));
    *ba = float(u);
    *bb = float(w);
}

// Points-to-mesh projection (MRMesh/MRPointsToMeshProjector.cpp:17-32 over MRMeshProject.cpp:13-104;
// the GPU counterpart is MRCuda/MRCudaPointsToMeshProjector.cu:6-111).  Each point is mapped by pxf
// (when given), the packet search finds the nearest triangle (FP32, FP64 near the surface in
// precise mode), and the winner's projection, barycentrics and distance are recomputed in FP64 and
// rounded as the reference CPU does.  Output per point, the layout of MR::MeshProjectionResult:
// {face, proj.xyz} {edge = -1, bary a, bary b, distSq}; face = -1 when nothing lies closer than up.
template <bool PRECISE, bool TREEXF>
__global__ void __launch_bounds__(kThreads, kDistBlocks) projectKernel(QueryTree t, const float* __restrict__ pts, int64_t n, Xf pxf,
                                                          int hasPxf, Xf txf, float up, float lo, float4* __restrict__ out,
                                                          unsigned* scratch, const int32_t* __restrict__ order, int chunk) {
    const int lane = threadIdx.x & 31;
    const uint64_t numTiles = (uint64_t(n) + 31) / 32;
    for (;;) {
        const unsigned item = nextTicket(scratch, lane);
        if (uint64_t(item) * chunk >= numTiles) break;
        int seed = -1;  // leaf slot closest to this lane's previous point (see vectorKernel)
        for (int jt = 0; jt < chunk; ++jt) {
            const uint64_t tile = uint64_t(item) * chunk + jt;
            if (tile >= numTiles) break;
            const int64_t r = int64_t(tile) * 32 + lane;
            const bool active = r < n;
            const int64_t i = (order && active) ? int64_t(order[r]) : r;
            float3 q = make_float3(0.f, 0.f, 0.f);
            if (active) {
                q = make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
                if (hasPxf) q = xfApply(pxf, q.x, q.y, q.z);
            }
            // start from the previous point's triangle when it lies within the limit: its distance is
            // one the search would reach anyway, so the minimum and the reported face are unchanged
            float upS = up;
            bool seeded = false;
            if (active && seed >= 0) {
                const float4* tr = t.tri + 3 * int64_t(seed);
                float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
                if (TREEXF) {
                    xfTri(&txf, A, B, C);
                }
                const float ds = triDistSq<PRECISE>(q, A, B, C);
                if (ds < upS) {
                    upS = ds;
                    seeded = true;
                }
            }
            int best = seeded ? seed : -1;
            const float dsq = cpPacket<PRECISE, true, TREEXF>(t, q, active, upS, lo, scratch + 1, &best, &txf);
            seed = best;
            if (!active) best = -2;
            float4 o0 = make_float4(__int_as_float(-1), 0.f, 0.f, 0.f), o1 = make_float4(__int_as_float(-1), 0.f, 0.f, dsq);
            if (best >= 0) {
                const float4* tr = t.tri + 3 * int64_t(best);
                float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
                if (TREEXF) {
                    xfTri(&txf, A, B, C);
                }
                float3 pr;
                float ba, bb;
                closestPointBaryFp64(q, A, B, C, &pr, &ba, &bb);
                const float dx = pr.x - q.x, dy = pr.y - q.y, dz = pr.z - q.z;
                o0 = make_float4(A.w, pr.x, pr.y, pr.z);
                o1 = make_float4(__int_as_float(-1), ba, bb, dot3rn(dx, dy, dz, dx, dy, dz));
            }
            if (active) {
                out[2 * i] = o0;
                out[2 * i + 1] = o1;
            }
        }
    }
}

// MRMesh/MRFastWindingNumber.cpp:40-52: query = triCenter(f) = (1/3) * (v0 + v1 + v2), skipping f.
// Lanes take consecutive leaf slots, which are spatially coherent.
template <bool PRECISE>
__global__ void __launch_bounds__(kThreads, 4) selfIntKernel(QueryTree t, float beta, uint64_t* __restrict__ bits,
                                                          float* __restrict__ wn, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const float betaSq = __fmul_rn(beta, beta);
    const uint64_t numTiles = (uint64_t(t.nLeaves) + 31) / 32;
    const bool rays = t.closed != 0 && beta >= 2.f && !wn;  // see below
    for (;;) {
        const unsigned tile = nextTicket(scratch, lane);
        if (tile >= numTiles) break;
        const int slot = int(tile) * 32 + lane;
        const bool active = slot < t.nLeaves;
        float3 q = make_float3(0.f, 0.f, 0.f);
        int face = -1;
        if (active) {
            const float4* tr = t.tri + 3 * int64_t(slot);
            const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
            const float third = 1 / 3.0f;
            q = make_float3(__fmul_rn(third, __fadd_rn(__fadd_rn(A.x, B.x), C.x)),
                            __fmul_rn(third, __fadd_rn(__fadd_rn(A.y, B.y), C.y)),
                            __fmul_rn(third, __fadd_rn(__fadd_rn(A.z, B.z), C.z)));
            face = __float_as_int(A.w);
        }
        // Closed surfaces, bits only: the ray from the centroid that ignores its own face counts the
        // exact winding number on the side of the face the ray leaves into; the other side differs by
        // one, by the face's orientation.  The reference's value (its own face skipped) lies halfway,
        // so the face is flagged when the smaller side is <= -1 or >= 1.  A face whose centroid does
        // not fall strictly inside its own projection (near-vertical or degenerate), or that lies on
        // another face, gets the approximated winding number as before.
        bool fwn = active, flag = false;
        if (rays) {
            int orient = 0;  // the sign of the face normal's z, exact
            if (active) {
                const float4* tr = t.tri + 3 * int64_t(slot);
                const float4 A = ld4(tr), B = ld4(tr + 1), C = ld4(tr + 2);
                const float ax = __fsub_rn(A.x, q.x), ay = __fsub_rn(A.y, q.y), bx = __fsub_rn(B.x, q.x),
                            by = __fsub_rn(B.y, q.y), cx = __fsub_rn(C.x, q.x), cy = __fsub_rn(C.y, q.y);
                const int e0 = edgeSign(bx, by, cx, cy), e1 = edgeSign(cx, cy, ax, ay), e2 = edgeSign(ax, ay, bx, by);
                if (e0 != 0 && e0 == e1 && e1 == e2) orient = e0;
            }
            bool onSurface = false, up = true;
            const int wd = rayWinding(t, q, active && orient != 0, scratch + 1, &onSurface, active ? slot : -1, &up);
            fwn = active && (orient == 0 || onSurface);
            if (active && !fwn) {
                const int a = up ? orient : -orient;  // +1: the face's normal points along the ray
                const int m = a > 0 ? wd : wd + a;    // the smaller of the two sides, wd and wd + a
                flag = m <= -1 || m >= 1;
            }
        }
        const float w = fwnPacket<PRECISE>(t, q, fwn, betaSq, active ? slot : -1, scratch + 1);
        if (active) {
            if (wn) wn[face] = w;
            if (fwn ? (w < 0.f || w > 1.f) : flag) atomicOr((unsigned long long*)bits + (face >> 6), 1ull << (face & 63));
        }
    }
}

__global__ void fillNan(float* p, int64_t n) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < n) p[i] = __int_as_float(0x7fc00000);
}

int gridBlocks(const void* kernel) {
    const int sms = numSMs();  // of the current device (an attribute query, cheap)
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, kThreads, 0);
    if (perSm < 1) perSm = 1;
    return sms * perSm;
}

template <typename K, typename... Args>
cudaError_t launchPersistent(K kernel, uint64_t work, unsigned* scratch, cudaStream_t s, Args... args) {
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned), s);
    if (e) return e;
    if (work == 0) return cudaSuccess;
    int blocks = gridBlocks((const void*)kernel);
    const uint64_t warpsNeeded = work;
    const uint64_t maxBlocks = (warpsNeeded + kThreads / 32 - 1) / (kThreads / 32);
    if (uint64_t(blocks) > maxBlocks) blocks = int(maxBlocks);
    kernel<<<blocks, kThreads, 0, s>>>(args...);
    return cudaGetLastError();
}

}  // namespace

int numSMs() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

uint64_t gridTiles(int32_t nx, int32_t ny, int32_t nz) {
    return uint64_t((nx + kTX - 1) / kTX) * uint64_t((ny + kTY - 1) / kTY) * uint64_t((nz + kTZ - 1) / kTZ);
}

static TileGrid tileGridFor(const GridRange& g, int maxSegLen = 16) {
    TileGrid tg;
    tg.tilesX = (g.nx + kTX - 1) / kTX;
    tg.tilesY = (g.ny + kTY - 1) / kTY;
    tg.tilesZ = (g.z1 - g.z0 + kTZ - 1) / kTZ;
    tg.numTiles = uint32_t(uint64_t(tg.tilesX) * tg.tilesY * tg.tilesZ);
    tg.runs = nullptr;
    tg.colState = nullptr;
    tg.signBits = nullptr;
    tg.fixList = nullptr;
    tg.fixCap = 0;
    // Longer columns reuse more seeds; shorter ones leave more items for the tail of the persistent
    // grid.  Measured at 256^3 / 512^3 on 1.3 M triangles: keep >= 25 items per (32-warps-per-SM)
    // resident warp, and columns of at most 32 tiles for unbanded signed distances (512^3: 16 tiles
    // +0.7 %, 64 +1 %) but 16 otherwise (banded requests, where the cost sits in the voxels near the
    // surface: 32 tiles made a 512^3 band 10 % slower).
    const uint64_t cols = uint64_t(tg.tilesX) * tg.tilesY;
    const uint64_t warps = uint64_t(numSMs()) * 4 * (kThreads / 32);
    tg.segLen = maxSegLen;
    while (tg.segLen > 1 && cols * uint64_t((tg.tilesZ + tg.segLen - 1) / tg.segLen) < 25 * warps) tg.segLen /= 2;
    tg.segsZ = (tg.tilesZ + tg.segLen - 1) / tg.segLen;
    tg.numItems = uint32_t(cols * tg.segsZ);
    return tg;
}

// Entries of the precise paired walk's fix list (after its counter): one per pair step at most.
static uint32_t pairFixCap(const TileGrid& tg) { return tg.numTiles / 2 + tg.numItems + 1; }

size_t pairFixBytes(uint32_t nTiles, uint32_t nItems) { return size_t(nTiles / 2 + nItems + 2) * sizeof(uint4); }
size_t pairFixBytesForRuns(int32_t nRuns, int32_t nBricks) {
    return pairFixBytes(uint32_t(nBricks) * 16u, uint32_t(nRuns) * uint32_t(kBrickCols));
}

// The signed distances of a grid (or of brick runs) with the column bits: the paired walk when there
// is no lower distance bound and the work items hold at least four tiles (in precise mode with its
// fix list, when given, and the fix-up pass), else the one-voxel walk.  Small grids get one-tile
// items (enough items for the persistent grid), which leave the pairs nothing to share: measured on
// the 1.31 M-triangle mesh, 128^3 4.8 ms one-voxel against 6.6 ms paired, 256^3 (4-tile items)
// 16.7 against 16.4 ms, 512^3 (32-tile items) 73.6 against 66.1 ms.
static cudaError_t launchWithBits(const QueryTree& t, const GridRange& g, TileGrid tg, const Xf& xf, const DistOpts& o, int precise,
                                  float* out, uint4* fix, unsigned* scratch, cudaStream_t s) {
    if (o.minDistSq <= 0.f && (tg.runs || tg.segLen >= 4) && (!precise || fix)) {
        if (!precise) return launchPersistent(gridPairKernel<false>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
        tg.fixList = fix;
        tg.fixCap = pairFixCap(tg);
        cudaError_t e = cudaMemsetAsync(fix, 0, sizeof(uint4), s);
        if (e || (e = launchPersistent(gridPairKernel<true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch))) return e;
        return launchPersistent(fixPairKernel, tg.fixCap, scratch, s, t, g, tg, xf, o, out, scratch);
    }
    if (precise) return launchPersistent(gridKernel<true, true, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
    return launchPersistent(gridKernel<false, true, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
}

cudaError_t launchGridSdfBricks(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o, int precise,
                                float* out, const int4* runs, int32_t nRuns, int32_t nBricks, const uint32_t* signBits,
                                void* fix, unsigned* scratch, cudaStream_t s) {
    TileGrid tg = tileGridFor(g);
    tg.runs = runs;
    tg.numTiles = uint32_t(nBricks) * 16u;
    tg.numItems = uint32_t(nRuns) * uint32_t(kBrickCols);
    if (signBits) {
        tg.signBits = signBits;
        return launchWithBits(t, g, tg, xf, o, precise, out, static_cast<uint4*>(fix), scratch, s);
    }
    if (precise)
        return launchPersistent(gridKernel<true, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
    return launchPersistent(gridKernel<false, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
}

bool signColumnsApply(const QueryTree& t, const Xf& xf, float beta, float threshold) {
    const float fr = threshold - floorf(threshold);
    // the (x, y) map must be well conditioned: the raster pass maps triangle bounds back to columns
    // through its inverse, in FP32
    const double det = double(xf.a[0]) * xf.a[4] - double(xf.a[1]) * xf.a[3];
    const double scale = (std::fabs(double(xf.a[0])) + std::fabs(double(xf.a[1]))) * (std::fabs(double(xf.a[3])) + std::fabs(double(xf.a[4])));
    return t.closed && beta >= 2.f && fr > 0.25f && fr < 0.75f && xf.a[2] == 0.f && xf.a[5] == 0.f && xf.a[8] > 0.f &&
           std::fabs(det) >= 1e-6 * scale && std::fabs(det) > 1e-30 && scale < 1e30;
}

size_t signColumnsWorkBytes(const GridRange& g) {
    const size_t ncols = size_t(g.nx) * size_t(g.ny);
    return ((2 * sizeof(uint32_t) + kColumnSlots * sizeof(float2)) * ncols + 255) & ~size_t(255);
}

cudaError_t launchSignColumns(const QueryTree& t, const GridRange& g, const Xf& xf, float beta, float threshold, int precise,
                              uint32_t* bits, float* values, void* work, size_t workBytes, unsigned* scratch, cudaStream_t s) {
    ColumnLists cl{};
    const size_t ncols = size_t(g.nx) * size_t(g.ny);
    if (work && workBytes >= signColumnsWorkBytes(g) && t.nLeaves > 0) {
        // zz first (8-byte aligned), then the counts and sign masks, cleared together
        cl.zz = static_cast<float2*>(work);
        cl.count = reinterpret_cast<uint32_t*>(cl.zz + kColumnSlots * ncols);
        cl.signMask = cl.count + ncols;
        cl.ncols = int64_t(ncols);
        const double a0 = xf.a[0], a1 = xf.a[1], a3 = xf.a[3], a4 = xf.a[4], det = a0 * a4 - a1 * a3;
        cl.inv[0] = float(a4 / det);
        cl.inv[1] = float(-a1 / det);
        cl.inv[2] = float(-a3 / det);
        cl.inv[3] = float(a0 / det);
        cl.org[0] = xf.b[0];
        cl.org[1] = xf.b[1];
        // xfPoint's four roundings of x = a0 i + a1 j + 0 k + b0: at most 2 ulps of the largest magnitude
        const auto margin = [](double m) { return float(4.0 * std::ldexp(1.0, std::ilogb(m > 0 ? m : 1e-30) - 23)); };
        cl.ex = margin(std::fabs(a0) * (g.nx - 1) + std::fabs(a1) * (g.ny - 1) + std::fabs(double(xf.b[0])));
        cl.ey = margin(std::fabs(a3) * (g.nx - 1) + std::fabs(a4) * (g.ny - 1) + std::fabs(double(xf.b[1])));
        cudaError_t e = cudaMemsetAsync(cl.count, 0, 2 * sizeof(uint32_t) * ncols, s);
        if (e) return e;
        int blocks = int(std::min<int64_t>((int64_t(t.nLeaves) + kThreads - 1) / kThreads, int64_t(numSMs()) * 16));
        columnRasterKernel<<<blocks, kThreads, 0, s>>>(t, g, xf, cl);
        if ((e = cudaGetLastError())) return e;
    }
    const uint64_t items = uint64_t((g.nx + 31) / 32) * uint64_t(g.ny) * uint64_t((g.z1 - g.z0 + kColumnSeg - 1) / kColumnSeg);
    if (precise)
        return launchPersistent(signColumnsKernel<true>, items, scratch, s, t, g, xf, threshold, beta, bits, values, cl, scratch);
    return launchPersistent(signColumnsKernel<false>, items, scratch, s, t, g, xf, threshold, beta, bits, values, cl, scratch);
}

cudaError_t launchGridFwn(const QueryTree& t, const GridRange& g, const Xf& xf, float beta, int precise, float* out,
                          unsigned* scratch, cudaStream_t s) {
    const TileGrid tg = tileGridFor(g);
    if (tg.segLen >= 2) {  // work items of two or more tiles: the paired walk
        if (precise) return launchPersistent(gridFwnPairKernel<true>, tg.numItems, scratch, s, t, g, tg, xf, beta, out, scratch);
        return launchPersistent(gridFwnPairKernel<false>, tg.numItems, scratch, s, t, g, tg, xf, beta, out, scratch);
    }
    DistOpts o{0.f, FLT_MAX, 0, 0.5f, beta};
    if (precise)
        return launchPersistent(gridKernel<true, false>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
    return launchPersistent(gridKernel<false, false>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
}

// Column hand-over words, then (when the column rays apply) the inside bits of the range.
size_t signBitsBytes(const GridRange& g) {
    return size_t((g.nx + 31) >> 5) * size_t(g.ny) * size_t(g.z1 - g.z0) * sizeof(uint32_t);
}

size_t gridSdfColumnStateBytes(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o) {
    const TileGrid tg = tileGridFor(g, o.maxDistSq >= FLT_MAX ? 32 : 16);
    const size_t col = size_t(tg.numItems) * (2 * kLayer) * sizeof(float);
    if (!signColumnsApply(t, xf, o.beta, o.threshold)) return col;
    return col + ((signBitsBytes(g) + 255) & ~size_t(255)) + signColumnsWorkBytes(g) +
           (o.minDistSq <= 0.f ? pairFixBytes(tg.numTiles, tg.numItems) : 0);
}


cudaError_t launchGridSdf(const QueryTree& t, const GridRange& g, const Xf& xf, const DistOpts& o, int precise, float* out,
                          unsigned* scratch, cudaStream_t s, float* colState, size_t colBytes) {
    TileGrid tg = tileGridFor(g, o.maxDistSq >= FLT_MAX ? 32 : 16);
    const size_t need = size_t(tg.numItems) * (2 * kLayer) * sizeof(float);
    if (colState && colBytes >= need && need > 0) {
        cudaError_t e = cudaMemsetAsync(colState, 0xff, need, s);
        if (e) return e;
        tg.colState = colState;
        if (signColumnsApply(t, xf, o.beta, o.threshold) && colBytes >= need + signBitsBytes(g)) {
            // closed surface, vertical z axis: the signs from the columns' crossings first
            char* base = reinterpret_cast<char*>(colState);
            uint32_t* bits = reinterpret_cast<uint32_t*>(base + need);
            const size_t lists = need + ((signBitsBytes(g) + 255) & ~size_t(255));
            void* work = colBytes >= lists + signColumnsWorkBytes(g) ? base + lists : nullptr;
            if ((e = launchSignColumns(t, g, xf, o.beta, o.threshold, precise, bits, nullptr, work, work ? colBytes - lists : 0,
                                       scratch, s)))
                return e;
            tg.signBits = bits;
            const size_t fixAt = lists + signColumnsWorkBytes(g);
            uint4* fix = (work && colBytes >= fixAt + pairFixBytes(tg.numTiles, tg.numItems))
                             ? reinterpret_cast<uint4*>(base + fixAt)
                             : nullptr;
            return launchWithBits(t, g, tg, xf, o, precise, out, fix, scratch, s);
        }
    }
    if (precise)
        return launchPersistent(gridKernel<true, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
    return launchPersistent(gridKernel<false, true>, tg.numItems, scratch, s, t, g, tg, xf, o, out, scratch);
}

// Tiles of 32 points per work item for the seeded point searches: only with a spatial order, and
// while at least 32 items per resident warp remain.  Morton-ordered point sets can hold long runs of
// expensive queries (points far from the surface), so the work items must stay small: with 5 M
// points (4 M near the surface, 1 M spread over the box) and 4 tiles per item the projection took
// 11.8 ms instead of 9.2 ms; at that size the rule below keeps one tile per item.
static int pointChunk(uint64_t tiles, const int32_t* order) {
    if (!order) return 1;
    const uint64_t warps = uint64_t(numSMs()) * 4 * (kThreads / 32);
    int k = 8;
    while (k > 1 && (tiles + k - 1) / k < 32 * warps) k /= 2;
    return k;
}

cudaError_t launchVectorFwn(const QueryTree& t, const float* pts, int64_t n, float beta, int32_t skipFace, int precise,
                            float* out, unsigned* scratch, cudaStream_t s, const int32_t* order) {
    DistOpts o{0.f, FLT_MAX, 0, 0.5f, beta};
    const uint64_t tiles = (uint64_t(n) + 31) / 32;
    if (order && skipFace < 0) {  // spatially ordered points, no face skipped: two tiles per walk
        const uint64_t pairs = (tiles + 1) / 2;
        if (precise) return launchPersistent(vectorFwnPairKernel<true>, pairs, scratch, s, t, pts, n, beta, out, scratch, order);
        return launchPersistent(vectorFwnPairKernel<false>, pairs, scratch, s, t, pts, n, beta, out, scratch, order);
    }
    if (precise)
        return launchPersistent(vectorKernel<true, false>, tiles, scratch, s, t, pts, n, o, skipFace, out, scratch, order, 1);
    return launchPersistent(vectorKernel<false, false>, tiles, scratch, s, t, pts, n, o, skipFace, out, scratch, order, 1);
}

cudaError_t launchVectorSdf(const QueryTree& t, const float* pts, int64_t n, const DistOpts& o, int precise, float* out,
                            unsigned* scratch, cudaStream_t s, const int32_t* order) {
    const uint64_t tiles = (uint64_t(n) + 31) / 32;
    const int k = pointChunk(tiles, order);
    const uint64_t items = (tiles + k - 1) / k;
    if (precise) return launchPersistent(vectorKernel<true, true>, items, scratch, s, t, pts, n, o, -1, out, scratch, order, k);
    return launchPersistent(vectorKernel<false, true>, items, scratch, s, t, pts, n, o, -1, out, scratch, order, k);
}

cudaError_t launchProject(const QueryTree& t, const float* pts, int64_t n, const Xf* pointXf, const Xf* treeXf, float upSq,
                          float loSq, int precise, float4* out, unsigned* scratch, cudaStream_t s, const int32_t* order) {
    const uint64_t tiles = (uint64_t(n) + 31) / 32;
    const int k = pointChunk(tiles, order);
    const uint64_t items = (tiles + k - 1) / k;
    const Xf id{{1, 0, 0, 0, 1, 0, 0, 0, 1}, {0, 0, 0}};
    const Xf px = pointXf ? *pointXf : id, tx = treeXf ? *treeXf : id;
    const int hp = pointXf ? 1 : 0;
    if (treeXf) {
        if (precise)
            return launchPersistent(projectKernel<true, true>, items, scratch, s, t, pts, n, px, hp, tx, upSq, loSq, out, scratch, order, k);
        return launchPersistent(projectKernel<false, true>, items, scratch, s, t, pts, n, px, hp, tx, upSq, loSq, out, scratch, order, k);
    }
    if (precise)
        return launchPersistent(projectKernel<true, false>, items, scratch, s, t, pts, n, px, hp, tx, upSq, loSq, out, scratch, order, k);
    return launchPersistent(projectKernel<false, false>, items, scratch, s, t, pts, n, px, hp, tx, upSq, loSq, out, scratch, order, k);
}

cudaError_t launchSelfIntersections(const QueryTree& t, float beta, int precise, uint64_t* bits, float* wn,
                                    unsigned* scratch, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bits, 0, sizeof(uint64_t) * size_t((t.nFaces + 63) / 64), s);
    if (e) return e;
    if (wn && t.nFaces > 0) {
        fillNan<<<unsigned((t.nFaces + 255) / 256), 256, 0, s>>>(wn, t.nFaces);
        if ((e = cudaGetLastError())) return e;
    }
    const uint64_t tiles = (uint64_t(t.nLeaves) + 31) / 32;
    if (precise) return launchPersistent(selfIntKernel<true>, tiles, scratch, s, t, beta, bits, wn, scratch);
    return launchPersistent(selfIntKernel<false>, tiles, scratch, s, t, beta, bits, wn, scratch);
}

// ------------------------------------------------------------------ batched meshes
// Many meshes, each with its own grid, in one persistent launch: the tiles of all grids form one
// ticket sequence (item i owns tickets [tileBase_i, tileBase_{i+1})); a warp takes a ticket, finds
// its item by binary search, and runs the same packet traversals on that item's tree.  Items are
// ordered by estimated cost, most expensive first, so the long grids start early and the short
// ones fill the tail.  Tile shape (TX x TY x TZ = 32 voxels) and block size are template
// parameters chosen by the autotuner.
namespace {

template <bool PRECISE, int TX, int TY, int TZ, int THREADS>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) batchKernel(const BatchItem* __restrict__ items, int nItems, uint32_t totalTiles,
                                                       unsigned* scratch) {
    static_assert(TX * TY * TZ == 32, "one voxel per lane");
    const int lane = threadIdx.x & 31;
    const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / (TX * TY);
    for (;;) {
        const unsigned ticket = nextTicket(scratch, lane);
        if (ticket >= totalTiles) break;
        int lo = 0, hi = nItems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].tileBase <= ticket) lo = mid; else hi = mid - 1;
        }
        // the item (tree, grid, transform, options: ~210 bytes) is staged in this warp's shared-memory
        // slot and read from there, instead of living in registers for the whole column walk
        // (measured 78.1 -> 74.9 ms on the 64-mesh batch)
        __shared__ BatchItem sItem[THREADS / 32];
        BatchItem& it = sItem[threadIdx.x >> 5];
        {
            static_assert(sizeof(BatchItem) % 4 == 0, "copied as 32-bit words");
            const uint32_t* src = reinterpret_cast<const uint32_t*>(items + lo);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&it);
            __syncwarp();  // every lane is done with the previous item
            for (int k = lane; k < int(sizeof(BatchItem) / 4); k += 32) dst[k] = src[k];
            __syncwarp();
        }
        // a ticket is a column of up to kBatchSeg tiles along z, walked upwards with each lane's
        // closest-point search seeded by its previous voxel's triangle (as gridKernel does)
        const unsigned local = ticket - it.tileBase;
        const int tilesX = (it.g.nx + TX - 1) / TX, tilesY = (it.g.ny + TY - 1) / TY;
        const int tx = int(local % unsigned(tilesX));
        const unsigned rest = local / unsigned(tilesX);
        const int ty = int(rest % unsigned(tilesY)), seg = int(rest / unsigned(tilesY));
        const int x = tx * TX + lx, y = ty * TY + ly;
        const QueryTree& t = it.t;  // read through the cache, not copied into registers
        const DistOpts o = it.o;
        const bool reuseOk = signReuseAllowed(t, o);
        int seed = -1;
        float below = __int_as_float(0x7fc00000);  // the preceding voxel's signed squared distance (gridKernel)
        for (int j = 0; j < kBatchSeg; ++j) {
            const int z0 = (seg * kBatchSeg + j) * TZ;
            if (z0 >= it.g.nz) break;
            const int z = z0 + lz;
            const bool active = x < it.g.nx && y < it.g.ny && z < it.g.nz;
            const float3 q = xfPoint(it.xf, x, y, z);
            float up = o.maxDistSq;
            if (active && seed >= 0) {
                const float4* tr = t.tri + 3 * int64_t(seed);
                const float ds = triDistSq<PRECISE>(q, ld4(tr), ld4(tr + 1), ld4(tr + 2));
                if (ds < up) up = ds;
            }
            int best = active ? seed : -1;
            const float dsq = cpPacket<PRECISE, true>(t, q, active, up, o.minDistSq, scratch + 1, &best);
            const bool valid = !(o.nullOutsideMinMax && (dsq < o.minDistSq || dsq >= o.maxDistSq));
            const bool complete = active && valid && dsq >= o.minDistSq;
            bool reIn = false;
            const bool reuse = reuseOk && reuseSign<TX, TY, TZ>(it.xf, x, y, z, z - (lz == 0 ? 1 : TZ), lz, q, below, complete,
                                                                dsq, &reIn);
            bool onSurface = false;  // as gridKernel: ray crossings on closed surfaces
            const int cw = reuseOk ? rayWinding(t, q, active && valid && !reuse, scratch + 1, &onSurface) : 0;
            const bool fwn = reuseOk ? onSurface : (active && valid);
            const float w = fwnPacket<PRECISE>(t, q, fwn, __fmul_rn(o.beta, o.beta), -1, scratch + 1);
            const bool inside = reuse ? reIn : (fwn ? w > o.threshold : float(cw) > o.threshold);
            const float d = __fsqrt_rn(dsq);
            const float res = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
            if (active) it.out[(size_t(z) * it.g.ny + y) * it.g.nx + x] = res;
            // the bottom layer's lanes continue from the voxel one layer below (as gridKernel does)
            const int src = lane + (TZ - 1) * TX * TY * (lz == 0);
            seed = __shfl_sync(FULL, best, src);
            below = __shfl_sync(FULL, complete ? (inside ? -dsq : dsq) : __int_as_float(0x7fc00000), src);
        }
    }
}

// The item of a ticket of a batched launch (binary search over the items' first tickets).
__device__ __forceinline__ int batchItemOf(const BatchItem* __restrict__ items, int nItems, unsigned ticket) {
    int lo = 0, hi = nItems - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (items[mid].tileBase <= ticket) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// batchKernel with the paired walk (gridPairKernel's): the column of a ticket two tiles at a time,
// each lane taking its voxel of the lower tile and the one TZ layers above through one packet walk
// (cpPacket2), then the lower voxel's sign and the upper one's from it (the voxel below each, as in
// batchKernel: sign reuse, rays, the winding-number walk).  Only for batches without a lower
// distance bound (minDistSq = 0 in every item).  In precise mode the walk runs in FP32 and the pair
// steps whose voxels came within a triangle's near-plane level are listed ({ticket, first tile, lane
// masks}) for fixBatchKernel.
template <bool PRECISE, int TX, int TY, int TZ, int THREADS>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) batchPairKernel(const BatchItem* __restrict__ items, int nItems,
                                                                           uint32_t totalTiles, uint4* fix, uint32_t fixCap,
                                                                           unsigned* scratch) {
    static_assert(TX * TY * TZ == 32, "one voxel per lane");
    static_assert(THREADS / 32 <= 8, "one sPairFix row per warp");
    const int lane = threadIdx.x & 31;
    const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / (TX * TY);
    for (;;) {
        const unsigned ticket = nextTicket(scratch, lane);
        if (ticket >= totalTiles) break;
        const int lo = batchItemOf(items, nItems, ticket);
        __shared__ BatchItem sItem[THREADS / 32];
        BatchItem& it = sItem[threadIdx.x >> 5];
        {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(items + lo);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&it);
            __syncwarp();
            for (int k = lane; k < int(sizeof(BatchItem) / 4); k += 32) dst[k] = src[k];
            __syncwarp();
        }
        const unsigned local = ticket - it.tileBase;
        const int tilesX = (it.g.nx + TX - 1) / TX, tilesY = (it.g.ny + TY - 1) / TY;
        const int tx = int(local % unsigned(tilesX));
        const unsigned rest = local / unsigned(tilesX);
        const int ty = int(rest % unsigned(tilesY)), seg = int(rest / unsigned(tilesY));
        const int x = tx * TX + lx, y = ty * TY + ly;
        const QueryTree& t = it.t;
        const DistOpts o = it.o;
        const bool reuseOk = signReuseAllowed(t, o);
        const bool vertical = it.xf.a[2] == 0.f && it.xf.a[5] == 0.f;
        const float betaSq = __fmul_rn(o.beta, o.beta);
        int seed = -1;
        float below = __int_as_float(0x7fc00000);
        for (int j = 0; j < kBatchSeg; j += 2) {
            const int zA0 = (seg * kBatchSeg + j) * TZ;
            if (zA0 >= it.g.nz) break;
            const bool hasB = j + 1 < kBatchSeg && zA0 + TZ < it.g.nz;
            const int za = zA0 + lz, zb = za + TZ;
            const bool inXY = x < it.g.nx && y < it.g.ny;
            const bool activeA = inXY && za < it.g.nz, activeB = inXY && hasB && zb < it.g.nz;
            const float3 qa = xfPoint(it.xf, x, y, za), qb = xfPoint(it.xf, x, y, zb);
            float ra = o.maxDistSq, rb = o.maxDistSq;
            int ba = -1, bb = -1;
            if (PRECISE) {
                if (lane == 0) sPairFix[threadIdx.x >> 5][0] = sPairFix[threadIdx.x >> 5][1] = 0u;
                __syncwarp();
            }
            if (seed >= 0 && (activeA || activeB)) {
                bool da = false, db = false;
                leafDist2<PRECISE>(t, seed, qa, qb, activeA, activeB, ra, rb, ba, bb, da, db);
            }
            cpPacket2<PRECISE>(t, qa, qb, activeA, activeB, ra, rb, ba, bb, scratch + 1, vertical);
            if (PRECISE) {
                __syncwarp();
                const unsigned ma = sPairFix[threadIdx.x >> 5][0], mb = sPairFix[threadIdx.x >> 5][1];
                if ((ma | mb) && lane == 0) {
                    const uint32_t k = atomicAdd(&fix[0].x, 1u);
                    if (k < fixCap) fix[1 + k] = make_uint4(ticket, uint32_t(j), ma, mb);
                }
            }
            const int src = lane + (TZ - 1) * TX * TY * (lz == 0);
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {  // the lower voxel's sign, then the upper one's from it
                const bool active = h ? activeB : activeA;
                if (h && !__any_sync(FULL, active)) break;
                const int z = h ? zb : za;
                const float3& q = h ? qb : qa;
                const float dsq = h ? rb : ra;
                const bool valid = !(o.nullOutsideMinMax && (dsq < o.minDistSq || dsq >= o.maxDistSq));
                const bool complete = active && valid && dsq >= o.minDistSq;
                bool reIn = false;
                const bool reuse = reuseOk && reuseSign<TX, TY, TZ>(it.xf, x, y, z, z - (lz == 0 ? 1 : TZ), lz, q, below, complete,
                                                                    dsq, &reIn);
                bool onSurface = false;
                const int cw = reuseOk ? rayWinding(t, q, active && valid && !reuse, scratch + 1, &onSurface) : 0;
                const bool fwn = reuseOk ? onSurface : (active && valid);
                const float w = fwnPacket<PRECISE>(t, q, fwn, betaSq, -1, scratch + 1);
                const bool inside = reuse ? reIn : (fwn ? w > o.threshold : float(cw) > o.threshold);
                const float d = __fsqrt_rn(dsq);
                if (active) it.out[(size_t(z) * it.g.ny + y) * it.g.nx + x] = valid ? (inside ? -d : d) : __int_as_float(0x7fc00000);
                below = __shfl_sync(FULL, complete ? (inside ? -dsq : dsq) : __int_as_float(0x7fc00000), src);
            }
            seed = __shfl_sync(FULL, hasB ? bb : ba, src);
        }
    }
}

// The listed pair steps of a precise batchPairKernel launch: each flagged voxel's closest distance by
// the precise walk, written with the sign its output already holds (decided by the sign pass, which
// the distance's last bits do not move for a voxel this close to the surface).
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(kThreads) fixBatchKernel(const BatchItem* __restrict__ items, int nItems, uint4* fix,
                                                           uint32_t fixCap, unsigned* scratch) {
    const int lane = threadIdx.x & 31;
    const int lx = lane % TX, ly = (lane / TX) % TY, lz = lane / (TX * TY);
    const uint32_t n = min(__ldcg(&fix[0].x), fixCap);
    for (;;) {
        const unsigned e = nextTicket(scratch, lane);
        if (e >= n) break;
        const uint4 f = fix[1 + e];
        const BatchItem& it = items[batchItemOf(items, nItems, f.x)];
        const unsigned local = f.x - it.tileBase;
        const int tilesX = (it.g.nx + TX - 1) / TX, tilesY = (it.g.ny + TY - 1) / TY;
        const unsigned rest = local / unsigned(tilesX);
        const int x = int(local % unsigned(tilesX)) * TX + lx, y = int(rest % unsigned(tilesY)) * TY + ly;
        const int seg = int(rest / unsigned(tilesY));
#pragma unroll 1
        for (int h = 0; h < 2; ++h) {
            const bool need = ((h ? f.w : f.z) >> lane) & 1u;
            if (!__any_sync(FULL, need)) continue;
            const int z = (seg * kBatchSeg + int(f.y) + h) * TZ + lz;
            const float3 q = xfPoint(it.xf, x, y, z);
            const float dsq = cpPacket<true>(it.t, q, need, it.o.maxDistSq, 0.f, scratch + 1);
            if (need) {
                float* p = it.out + (size_t(z) * it.g.ny + y) * it.g.nx + x;
                const float old = *p;
                const bool valid = !(it.o.nullOutsideMinMax && dsq >= it.o.maxDistSq);
                if (old == old && valid) *p = copysignf(__fsqrt_rn(dsq), old);
            }
        }
    }
}

template <bool PRECISE, int TX, int TY, int TZ, int THREADS>
cudaError_t launchBatchT(const BatchItem* items, int nItems, uint32_t totalTiles, unsigned* scratch, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned), s);
    if (e || totalTiles == 0) return e;
    auto* k = batchKernel<PRECISE, TX, TY, TZ, THREADS>;
    const int sms = numSMs();
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k, THREADS, 0);
    int blocks = sms * (perSm < 1 ? 1 : perSm);
    const uint64_t maxBlocks = (uint64_t(totalTiles) + THREADS / 32 - 1) / (THREADS / 32);
    if (uint64_t(blocks) > maxBlocks) blocks = int(maxBlocks);
    k<<<blocks, THREADS, 0, s>>>(items, nItems, totalTiles, scratch);
    return cudaGetLastError();
}

template <bool PRECISE, int TX, int TY, int TZ, int THREADS>
cudaError_t launchBatchPairT(const BatchItem* items, int nItems, uint32_t totalTiles, uint4* fix, uint32_t fixCap, unsigned* scratch,
                             cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned), s);
    if (!e && PRECISE) e = cudaMemsetAsync(fix, 0, sizeof(uint4), s);
    if (e || totalTiles == 0) return e;
    auto* k = batchPairKernel<PRECISE, TX, TY, TZ, THREADS>;
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k, THREADS, 0);
    int blocks = numSMs() * (perSm < 1 ? 1 : perSm);
    const uint64_t maxBlocks = (uint64_t(totalTiles) + THREADS / 32 - 1) / (THREADS / 32);
    if (uint64_t(blocks) > maxBlocks) blocks = int(maxBlocks);
    k<<<blocks, THREADS, 0, s>>>(items, nItems, totalTiles, fix, fixCap, scratch);
    if ((e = cudaGetLastError()) || !PRECISE) return e;
    return launchPersistent(fixBatchKernel<TX, TY, TZ>, fixCap, scratch, s, items, nItems, fix, fixCap, scratch);
}

template <bool PRECISE>
cudaError_t launchBatchP(const BatchItem* items, int nItems, uint32_t totalTiles, int config, unsigned* scratch,
                         cudaStream_t s) {
    switch (config) {
        case 0: return launchBatchT<PRECISE, 4, 4, 2, 256>(items, nItems, totalTiles, scratch, s);
        case 1: return launchBatchT<PRECISE, 4, 4, 2, 128>(items, nItems, totalTiles, scratch, s);
        case 2: return launchBatchT<PRECISE, 8, 4, 1, 256>(items, nItems, totalTiles, scratch, s);
        case 3: return launchBatchT<PRECISE, 8, 4, 1, 128>(items, nItems, totalTiles, scratch, s);
        case 4: return launchBatchT<PRECISE, 2, 4, 4, 256>(items, nItems, totalTiles, scratch, s);
        case 5: return launchBatchT<PRECISE, 2, 4, 4, 128>(items, nItems, totalTiles, scratch, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

template <bool PRECISE>
cudaError_t launchBatchPairP(const BatchItem* items, int nItems, uint32_t totalTiles, int config, uint4* fix, uint32_t fixCap,
                             unsigned* scratch, cudaStream_t s) {
    switch (config) {
        case 0: return launchBatchPairT<PRECISE, 4, 4, 2, 256>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 1: return launchBatchPairT<PRECISE, 4, 4, 2, 128>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 2: return launchBatchPairT<PRECISE, 8, 4, 1, 256>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 3: return launchBatchPairT<PRECISE, 8, 4, 1, 128>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 4: return launchBatchPairT<PRECISE, 2, 4, 4, 256>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        case 5: return launchBatchPairT<PRECISE, 2, 4, 4, 128>(items, nItems, totalTiles, fix, fixCap, scratch, s);
        default: return cudaErrorInvalidValue;
    }
}

const char* batchConfigName(int config) {
    static const char* names[kBatchConfigs] = {
        "tile 4x4x2, 256 threads",         "tile 4x4x2, 128 threads",         "tile 8x4x1, 256 threads",
        "tile 8x4x1, 128 threads",         "tile 2x4x4, 256 threads",         "tile 2x4x4, 128 threads",
        "tile 4x4x2, 256 threads, paired", "tile 4x4x2, 128 threads, paired", "tile 8x4x1, 256 threads, paired",
        "tile 8x4x1, 128 threads, paired", "tile 2x4x4, 256 threads, paired", "tile 2x4x4, 128 threads, paired"};
    return (config >= 0 && config < kBatchConfigs) ? names[config] : "";
}

uint64_t batchTiles(int config, int32_t nx, int32_t ny, int32_t nz) {
    static const int shape[kBatchShapes][3] = {{4, 4, 2}, {4, 4, 2}, {8, 4, 1}, {8, 4, 1}, {2, 4, 4}, {2, 4, 4}};
    const int* t = shape[(config >= 0 && config < kBatchConfigs) ? config % kBatchShapes : 0];
    const uint64_t tilesZ = uint64_t((nz + t[2] - 1) / t[2]);
    return uint64_t((nx + t[0] - 1) / t[0]) * uint64_t((ny + t[1] - 1) / t[1]) * ((tilesZ + kBatchSeg - 1) / kBatchSeg);
}

uint32_t batchFixCap(uint32_t totalTiles) {  // one entry per pair step at most (kept below 2^31 entries)
    return uint32_t(std::min<uint64_t>(uint64_t(totalTiles) * (kBatchSeg / 2) + 1, 0x7fffffffull));
}

cudaError_t launchBatchSdf(const BatchItem* items, int nItems, uint32_t totalTiles, int precise, int config, bool pairOk,
                           void* fix, unsigned* scratch, cudaStream_t s) {
    // a paired variant needs every item without a lower distance bound, and in precise mode the fix
    // list; otherwise it runs as its one-voxel counterpart (the same grids)
    if (config >= kBatchShapes && pairOk && (!precise || fix)) {
        uint4* f = static_cast<uint4*>(fix);
        const uint32_t cap = batchFixCap(totalTiles);
        if (precise) return launchBatchPairP<true>(items, nItems, totalTiles, config - kBatchShapes, f, cap, scratch, s);
        return launchBatchPairP<false>(items, nItems, totalTiles, config - kBatchShapes, f, cap, scratch, s);
    }
    if (precise) return launchBatchP<true>(items, nItems, totalTiles, config % kBatchShapes, scratch, s);
    return launchBatchP<false>(items, nItems, totalTiles, config % kBatchShapes, scratch, s);
}

}  // namespace gbfwn
