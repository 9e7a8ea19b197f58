#pragma once
// Traversal primitives shared by the query translation units (query.cu, columns.cu): the reference
// arithmetic helpers, the packet walks (winding number, closest point, paired forms, vertical rays),
// the tile constants and the persistent-launch helpers.  Everything here has internal linkage: each
// translation unit compiles its own copy.
//
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
}  // namespace gbfwn
