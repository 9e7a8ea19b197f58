// Tree and dipole construction.
//
// The tree must be the reference's tree node for node: the far-field decisions of the winding
// number (MRMesh/MRDipole.h:18-27) depend on how triangles are grouped, so any other tree gives
// different (equally approximate) winding numbers.  The reference builds it by recursive median
// splits (MRMesh/MRAABBTreeMaker.hpp:51-165): the leaves of a node are ordered by the box-centre
// coordinate (min + max) along the node box's largest dimension, then the second largest, then
// the smallest, then by face id; the first floor(n/2) go left; nodes are stored in pre-order.
// Because that order is total, the split sets do not depend on how the partition is computed.
//
// This file is compiled with -fmad=false: every float expression below rounds each operation
// separately, exactly like the reference's CPU code, so dipoles and radii are bit-identical to the
// reference's.  The tree topology itself is built on the device by treebuild.cu.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "common.cuh"

namespace gbfwn {

// ------------------------------------------------------------------------------------ device
namespace {

__device__ __forceinline__ float3 vload(const float* v, int i) { return make_float3(v[3 * i], v[3 * i + 1], v[3 * i + 2]); }

// MRMesh/MRDipole.cpp:29-44 leaf dipoles: pos = area * triCenter, area = |dirArea|,
// dirArea = 0.5 * cross(b - a, c - a) (MRMesh/MRMeshMath.cpp:119-124,140-149).
__global__ void leafDipolesKernel(const RefNode* __restrict__ nodes, int64_t nNodes, const float* __restrict__ verts,
                                  const int32_t* __restrict__ tris, float* __restrict__ dip8, int* __restrict__ arrive) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    arrive[i] = 0;
    const RefNode nd = nodes[i];
    float* d = dip8 + 8 * i;
    if (nd.r >= 0) return;
    const int32_t* t = tris + 3 * int64_t(nd.l);
    const float3 a = vload(verts, t[0]), b = vload(verts, t[1]), c = vload(verts, t[2]);
    const float3 ab = make_float3(b.x - a.x, b.y - a.y, b.z - a.z);
    const float3 ac = make_float3(c.x - a.x, c.y - a.y, c.z - a.z);
    const float3 da = make_float3(0.5f * (ab.y * ac.z - ab.z * ac.y), 0.5f * (ab.z * ac.x - ab.x * ac.z),
                                  0.5f * (ab.x * ac.y - ab.y * ac.x));
    const float area = sqrtf(da.x * da.x + da.y * da.y + da.z * da.z);
    const float third = 1 / 3.0f;
    const float3 ctr = make_float3(third * (a.x + b.x + c.x), third * (a.y + b.y + c.y), third * (a.z + b.z + c.z));
    d[0] = area * ctr.x;
    d[1] = area * ctr.y;
    d[2] = area * ctr.z;
    d[3] = area;
    d[4] = da.x;
    d[5] = da.y;
    d[6] = da.z;
    d[7] = 0;
}

__global__ void parentsKernel(const RefNode* __restrict__ nodes, int64_t nNodes, int32_t* __restrict__ parent) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    if (i == 0) parent[0] = -1;
    const RefNode nd = nodes[i];
    if (nd.r < 0) return;
    parent[nd.l] = int32_t(i);
    parent[nd.r] = int32_t(i);
}

// MRMesh/MRDipole.cpp:47-60: internal dipole = left + right (pos and dirArea are still
// area-weighted sums here).  Each leaf thread climbs; the second child to arrive at a parent
// computes it.  dl + dr is commutative, so the result is the reference's whatever arrives first.
// The children's 32-byte rows are read from L2 (ld.global.cg, past this SM's L1, which may hold a
// row from before the sibling's thread wrote it) as two 16-byte loads.
__global__ void sumUpKernel(const RefNode* __restrict__ nodes, int64_t nNodes, const int32_t* __restrict__ parent,
                            float* dip8, int* arrive) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    if (nodes[i].r >= 0) return;
    int32_t p = parent[i];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&arrive[p], 1) == 0) return;  // first arrival: the sibling's thread finishes p
        __threadfence();
        const RefNode nd = nodes[p];
        const float4* dl = reinterpret_cast<const float4*>(dip8 + 8 * int64_t(nd.l));
        const float4* dr = reinterpret_cast<const float4*>(dip8 + 8 * int64_t(nd.r));
        const float4 l0 = __ldcg(dl), l1 = __ldcg(dl + 1), r0 = __ldcg(dr), r1 = __ldcg(dr + 1);
        float4* d = reinterpret_cast<float4*>(dip8 + 8 * int64_t(p));
        d[0] = make_float4(l0.x + r0.x, l0.y + r0.y, l0.z + r0.z, l0.w + r0.w);
        d[1] = make_float4(l1.x + r1.x, l1.y + r1.y, l1.z + r1.z, 0.f);
        p = parent[p];
    }
}

// MRMesh/MRDipole.cpp:63-70 + 11-21: centre of mass and squared distance to the farthest box corner.
__global__ void finalizeKernel(const RefNode* __restrict__ nodes, int64_t nNodes, float* __restrict__ dip8) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    float* d = dip8 + 8 * i;
    float px = d[0], py = d[1], pz = d[2];
    const float area = d[3];
    if (area > 0) {
        const float inv = 1 / area;
        px = px * inv;
        py = py * inv;
        pz = pz * inv;
    }
    const RefNode nd = nodes[i];
    const float mn[3] = {nd.minx, nd.miny, nd.minz}, mx[3] = {nd.maxx, nd.maxy, nd.maxz}, p[3] = {px, py, pz};
    float rr = 0;
    for (int k = 0; k < 3; ++k) {
        const float a = p[k] - mn[k], b = p[k] - mx[k];
        rr = rr + fmaxf(a * a, b * b);
    }
    d[0] = px;
    d[1] = py;
    d[2] = pz;
    d[7] = rr;
}

// Wide query records (layout in common.cuh).  irank[i] = internal index of node i (or -1),
// slot[i] = leaf slot of node i (or -1).
__device__ __forceinline__ int32_t linkOf(int32_t node, const int32_t* irank, const int32_t* slot) {
    const int32_t k = irank[node];
    return k >= 0 ? k : ~slot[node];
}

__global__ void packKernel(const RefNode* __restrict__ nodes, int64_t nNodes, const float* __restrict__ dip8,
                           const int32_t* __restrict__ irank, const int32_t* __restrict__ slot,
                           const float* __restrict__ verts, const int32_t* __restrict__ tris, float4* __restrict__ cp,
                           float4* __restrict__ dip, float4* __restrict__ tri, int32_t* __restrict__ faceSlot) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    const RefNode nd = nodes[i];
    if (nd.r < 0) {
        const int32_t s = slot[i];
        const int32_t* t = tris + 3 * int64_t(nd.l);
        const float3 a = vload(verts, t[0]), b = vload(verts, t[1]), c = vload(verts, t[2]);
        // b.w flags a triangle whose (x, y) projection has (next to) no area: vertical rays never
        // cross it, though a point of one may lie on it (the rays' on-surface rule)
        const float e1x = b.x - a.x, e1y = b.y - a.y, e2x = c.x - a.x, e2y = c.y - a.y;
        const float area2 = fmaf(e1x, e2y, -e1y * e2x);
        const float len2 = fmaf(e1x, e1x, e1y * e1y) + fmaf(e2x, e2x, e2y * e2y) + fmaf(c.x - b.x, c.x - b.x, (c.y - b.y) * (c.y - b.y));
        const float vertical = fabsf(area2) <= 1e-6f * len2 ? 1.f : 0.f;
        tri[3 * int64_t(s) + 0] = make_float4(a.x, a.y, a.z, __int_as_float(nd.l));
        tri[3 * int64_t(s) + 1] = make_float4(b.x, b.y, b.z, vertical);
        tri[3 * int64_t(s) + 2] = make_float4(c.x, c.y, c.z,
                                              nearPlaneLevel(make_float4(a.x, a.y, a.z, 0.f), make_float4(b.x, b.y, b.z, 0.f),
                                                             make_float4(c.x, c.y, c.z, 0.f)));
        faceSlot[nd.l] = s;
        return;
    }
    const int64_t k = irank[i];
    const int32_t ll = linkOf(nd.l, irank, slot), rl = linkOf(nd.r, irank, slot);
    (void)cp;
    const float* dl = dip8 + 8 * int64_t(nd.l);
    const float* dr = dip8 + 8 * int64_t(nd.r);
    dip[4 * k + 0] = make_float4(dl[0], dl[1], dl[2], dl[7]);
    dip[4 * k + 1] = make_float4(dl[4], dl[5], dl[6], __int_as_float(ll));
    dip[4 * k + 2] = make_float4(dr[0], dr[1], dr[2], dr[7]);
    dip[4 * k + 3] = make_float4(dr[4], dr[5], dr[6], __int_as_float(rl));
}

// Oriented bounding box of every non-root node, written into its parent's closest-point record
// (layout in common.cuh).  Both children of a node are boxed in the PARENT's frame: n = the parent's
// dipole direction dirArea (the area-weighted normal of its triangles), t and u completing an
// orthonormal basis, so a query projects itself once per record for both children.  Extents = the
// range of the projections of all the node's triangle vertices, widened by a relative margin that
// covers the FP32 rounding of the projections here and at query time, so the box distance stays a
// lower bound of the distance to every triangle inside.  The node's leaves are the contiguous slots
// range[i] = (first, count).  Nodes of up to kObbChunk leaves: obbKernel (a thread for a node of up
// to 4 leaves, a warp for a larger one); larger ones (the top levels, about 2n / kObbChunk nodes):
// one warp per chunk of kObbChunk leaves,
// combined with order-independent atomic min / max (obbChunkKernel), then written by
// obbBigKernel -- so no warp walks more than kObbChunk triangles.
constexpr int kObbChunk = 4096;

struct Frame {
    float t[3], u[3], n[3];
};

__device__ __forceinline__ Frame nodeFrame(const float* __restrict__ dip8, int64_t i) {
    const float* d = dip8 + 8 * i;
    float nx = d[4], ny = d[5], nz = d[6];
    const float len = sqrtf(nx * nx + ny * ny + nz * nz);
    if (!(len > 1e-30f)) {
        nx = 0.f; ny = 0.f; nz = 1.f;
    } else {
        nx /= len; ny /= len; nz /= len;
    }
    float ax = 1.f, ay = 0.f;
    if (fabsf(nx) > 0.6f) { ax = 0.f; ay = 1.f; }
    const float an = ax * nx + ay * ny;
    float tx = ax - an * nx, ty = ay - an * ny, tz = -an * nz;
    const float tl = sqrtf(tx * tx + ty * ty + tz * tz);
    tx /= tl; ty /= tl; tz /= tl;
    Frame f;
    f.t[0] = tx; f.t[1] = ty; f.t[2] = tz;
    f.u[0] = ny * tz - nz * ty; f.u[1] = nz * tx - nx * tz; f.u[2] = nx * ty - ny * tx;
    f.n[0] = nx; f.n[1] = ny; f.n[2] = nz;
    return f;
}

// lo / hi of the projections of the triangles in slots [a, b) (this lane's share), reduced over the warp
__device__ __forceinline__ void projRange(const Frame& f, const float4* __restrict__ tri, int a, int b, int lane, float lo[3],
                                          float hi[3]) {
    for (int j = 0; j < 3; ++j) {
        lo[j] = FLT_MAX;
        hi[j] = -FLT_MAX;
    }
    for (int sidx = a + lane; sidx < b; sidx += 32) {
        for (int k = 0; k < 3; ++k) {
            const float4 v = tri[3 * int64_t(sidx) + k];
            const float p[3] = {f.t[0] * v.x + f.t[1] * v.y + f.t[2] * v.z, f.u[0] * v.x + f.u[1] * v.y + f.u[2] * v.z,
                                f.n[0] * v.x + f.n[1] * v.y + f.n[2] * v.z};
            for (int j = 0; j < 3; ++j) {
                lo[j] = fminf(lo[j], p[j]);
                hi[j] = fmaxf(hi[j], p[j]);
            }
        }
    }
    for (int off = 16; off; off >>= 1)
        for (int j = 0; j < 3; ++j) {
            lo[j] = fminf(lo[j], __shfl_xor_sync(0xffffffffu, lo[j], off));
            hi[j] = fmaxf(hi[j], __shfl_xor_sync(0xffffffffu, hi[j], off));
        }
}

__device__ __forceinline__ void writeObb(int64_t i, const Frame& f, const float lo[3], const float hi[3],
                                         const int32_t* __restrict__ parent, const int32_t* __restrict__ irank,
                                         const int32_t* __restrict__ slot, float4* __restrict__ cp) {
    float c[3], e[3];
    for (int j = 0; j < 3; ++j) {
        c[j] = 0.5f * (lo[j] + hi[j]);
        const float h = 0.5f * (hi[j] - lo[j]);
        e[j] = h + 2e-6f * (fabsf(c[j]) + h) + 1e-30f;
    }
    const int32_t p = parent[i];
    const int side = (i == int64_t(p) + 1) ? 0 : 1;
    const int32_t k = irank[i];
    const int32_t link = k >= 0 ? k : ~slot[i];
    float4* dst = cp + 6 * int64_t(irank[p]);
    if (side == 0) {  // the left child also writes the (shared) frame
        dst[0] = make_float4(f.t[0], f.t[1], f.t[2], f.u[0]);
        dst[1] = make_float4(f.u[1], f.u[2], f.n[0], f.n[1]);
        dst[2] = make_float4(f.n[2], c[0], c[1], c[2]);
        dst[3] = make_float4(e[0], e[1], e[2], __int_as_float(link));
    } else {
        dst[4] = make_float4(c[0], c[1], c[2], e[0]);
        dst[5] = make_float4(e[1], e[2], __int_as_float(link), 0.f);
    }
}

// Nodes of up to kObbThread leaves (three quarters of all nodes): one thread each; larger ones up to
// kObbChunk leaves: the warp of the 32 consecutive nodes holding them, one node after the other.
// min / max are exact, so the boxes are the same however the projections are split.
constexpr int kObbThread = 4;

__global__ void obbKernel(int64_t nNodes, const float* __restrict__ dip8, const int2* __restrict__ range,
                          const float4* __restrict__ tri, const int32_t* __restrict__ parent,
                          const int32_t* __restrict__ irank, const int32_t* __restrict__ slot, float4* __restrict__ cp) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    const int lane = threadIdx.x & 31;
    int2 r = make_int2(0, 0);
    if (i < nNodes && i != 0) r = range[i];
    if (r.y >= 1 && r.y <= kObbThread) {
        const Frame f = nodeFrame(dip8, parent[i]);
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int sidx = r.x; sidx < r.x + r.y; ++sidx) {
            for (int k = 0; k < 3; ++k) {
                const float4 v = tri[3 * int64_t(sidx) + k];
                const float p[3] = {f.t[0] * v.x + f.t[1] * v.y + f.t[2] * v.z, f.u[0] * v.x + f.u[1] * v.y + f.u[2] * v.z,
                                    f.n[0] * v.x + f.n[1] * v.y + f.n[2] * v.z};
                for (int j = 0; j < 3; ++j) {
                    lo[j] = fminf(lo[j], p[j]);
                    hi[j] = fmaxf(hi[j], p[j]);
                }
            }
        }
        writeObb(i, f, lo, hi, parent, irank, slot, cp);
    }
    unsigned big = __ballot_sync(0xffffffffu, r.y > kObbThread && r.y <= kObbChunk);
    while (big) {  // obbChunkKernel / obbBigKernel take the nodes above kObbChunk
        const int src = __ffs(big) - 1;
        big &= big - 1;
        const int64_t j = i - lane + src;
        const int first = __shfl_sync(0xffffffffu, r.x, src), num = __shfl_sync(0xffffffffu, r.y, src);
        const Frame f = nodeFrame(dip8, parent[j]);
        float lo[3], hi[3];
        projRange(f, tri, first, first + num, lane, lo, hi);
        if (lane == 0) writeObb(j, f, lo, hi, parent, irank, slot, cp);
    }
}

// float <-> int with the same order (for atomicMin / atomicMax on signed ints)
__device__ __forceinline__ int orderedKey(float x) {
    const int b = __float_as_int(x);
    return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float orderedVal(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }

// chunks of the big nodes: chunkStart[i] = first chunk of node i (exclusive scan of its chunk count),
// big[i] = its index among the big nodes; acc = 6 ordered keys (lo xyz, hi xyz) per big node
__global__ void obbChunkCount(const int2* __restrict__ range, int64_t nNodes, int32_t* __restrict__ nChunks,
                              int32_t* __restrict__ isBig) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    const int cnt = range[i].y;
    const bool big = i > 0 && cnt > kObbChunk;
    nChunks[i] = big ? (cnt + kObbChunk - 1) / kObbChunk : 0;
    isBig[i] = big ? 1 : 0;
}

__global__ void obbAccInit(int* __restrict__ acc, const int32_t* __restrict__ nBig, int64_t maxBig) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= 6 * min(int64_t(*nBig), maxBig)) return;
    acc[i] = (i % 6) < 3 ? orderedKey(FLT_MAX) : orderedKey(-FLT_MAX);
}

__global__ void obbChunkKernel(int64_t nNodes, const float* __restrict__ dip8, const int2* __restrict__ range,
                               const float4* __restrict__ tri, const int32_t* __restrict__ chunkStart,
                               const int32_t* __restrict__ totalChunks, const int32_t* __restrict__ bigIdx,
                               int64_t maxBig, int* __restrict__ acc, const int32_t* __restrict__ parent) {
    const int lane = threadIdx.x & 31;
    const int64_t nWarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    const int total = *totalChunks;
    for (int64_t w = (blockIdx.x * int64_t(blockDim.x) + threadIdx.x) >> 5; w < total; w += nWarps) {
        int64_t lo_ = 0, hi_ = nNodes - 1;  // last node whose first chunk is <= w
        while (lo_ < hi_) {
            const int64_t mid = (lo_ + hi_ + 1) >> 1;
            if (chunkStart[mid] <= w) lo_ = mid; else hi_ = mid - 1;
        }
        const int64_t i = lo_;
        const int2 r = range[i];
        const int a = r.x + int(w - chunkStart[i]) * kObbChunk, b = min(a + kObbChunk, r.x + r.y);
        const Frame f = nodeFrame(dip8, parent[i]);
        float lo[3], hi[3];
        projRange(f, tri, a, b, lane, lo, hi);
        if (lane == 0 && bigIdx[i] < maxBig) {
            int* d = acc + 6 * int64_t(bigIdx[i]);
            for (int j = 0; j < 3; ++j) {
                atomicMin(d + j, orderedKey(lo[j]));
                atomicMax(d + 3 + j, orderedKey(hi[j]));
            }
        }
    }
}

__global__ void obbBigKernel(int64_t nNodes, const float* __restrict__ dip8, const int32_t* __restrict__ isBig,
                             const int32_t* __restrict__ bigIdx, int64_t maxBig, const int* __restrict__ acc,
                             const int32_t* __restrict__ parent, const int32_t* __restrict__ irank,
                             const int32_t* __restrict__ slot, float4* __restrict__ cp) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes || !isBig[i] || bigIdx[i] >= maxBig) return;
    const int* d = acc + 6 * int64_t(bigIdx[i]);
    const float lo[3] = {orderedVal(d[0]), orderedVal(d[1]), orderedVal(d[2])};
    const float hi[3] = {orderedVal(d[3]), orderedVal(d[4]), orderedVal(d[5])};
    writeObb(i, nodeFrame(dip8, parent[i]), lo, hi, parent, irank, slot, cp);
}

// ------------------------------------------------------------------------------------ refit
// MRMesh/MRAABBTree.cpp:62-94 AABBTree::refit: leaves whose face touches a changed vertex get the
// face box again (MRMesh/MRAABBTree.cpp:15-29 computeFaceBox, one ulp wider each way); every
// internal node above a changed node becomes the union of its children.  Internal boxes are
// recomputed here for all nodes: a node with no changed descendant already is that union, so the
// result is the reference's node for node.
__global__ void refitLeafKernel(RefNode* __restrict__ nodes, int64_t nNodes, const float* __restrict__ verts,
                                const int32_t* __restrict__ tris, const uint64_t* __restrict__ changed, int64_t nv,
                                int* __restrict__ arrive) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    arrive[i] = 0;
    const RefNode nd = nodes[i];
    if (nd.r >= 0) return;
    const int32_t* t = tris + 3 * int64_t(nd.l);
    if (changed) {
        bool any = false;
        for (int k = 0; k < 3; ++k) {
            const int64_t v = t[k];
            if (v >= 0 && v < nv && ((changed[v >> 6] >> (v & 63)) & 1ull)) any = true;
        }
        if (!any) return;
    }
    float mn[3], mx[3];
    for (int d = 0; d < 3; ++d) {
        float lo = FLT_MAX, hi = -FLT_MAX;
        for (int k = 0; k < 3; ++k) {
            const float x = verts[3 * int64_t(t[k]) + d];
            if (x < lo) lo = x;
            if (x > hi) hi = x;
        }
        mn[d] = nextafterf(lo, -FLT_MAX);
        mx[d] = nextafterf(hi, FLT_MAX);
    }
    nodes[i] = RefNode{mn[0], mn[1], mn[2], mx[0], mx[1], mx[2], nd.l, nd.r};
}

// internal boxes bottom-up: the second child to arrive at a parent writes the union (MRBox.h:132-139)
__global__ void refitUpKernel(RefNode* nodes, int64_t nNodes, const int32_t* __restrict__ parent, int* arrive) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    if (nodes[i].r >= 0) return;
    int32_t p = parent[i];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(&arrive[p], 1) == 0) return;
        __threadfence();
        // the links never change here; the children's boxes are read from L2 as in sumUpKernel
        const int32_t l = nodes[p].l, r = nodes[p].r;
        const float4* nl = reinterpret_cast<const float4*>(nodes + l);
        const float4* nr = reinterpret_cast<const float4*>(nodes + r);
        const float4 l0 = __ldcg(nl), l1 = __ldcg(nl + 1), r0 = __ldcg(nr), r1 = __ldcg(nr + 1);
        float a[6] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y}, b[6] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y};
        for (int k = 0; k < 3; ++k) {
            if (b[k] < a[k]) a[k] = b[k];
            if (b[3 + k] > a[3 + k]) a[3 + k] = b[3 + k];
        }
        nodes[p] = RefNode{a[0], a[1], a[2], a[3], a[4], a[5], l, r};
        p = parent[p];
    }
}

// internal rank, leaf slot and leaf range of every node from the pre-order layout alone:
// leafBefore = leaves before node i (exclusive scan of the leaf flags); a subtree's last leaf is
// reached by following right children.
__global__ void leafFlagKernel(const RefNode* __restrict__ nodes, int64_t nNodes, int32_t* __restrict__ flag) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < nNodes) flag[i] = nodes[i].r < 0 ? 1 : 0;
}

__global__ void ranksKernel(const RefNode* __restrict__ nodes, int64_t nNodes, const int32_t* __restrict__ leafBefore,
                            int32_t* __restrict__ irs, int2* __restrict__ range) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= nNodes) return;
    const int32_t first = leafBefore[i];
    if (nodes[i].r < 0) {
        irs[i] = -1;
        irs[nNodes + i] = first;
        range[i] = make_int2(first, 1);
        return;
    }
    int32_t last = nodes[i].r;
    while (nodes[last].r >= 0) last = nodes[last].r;
    irs[i] = int32_t(i) - first;
    irs[nNodes + i] = -1;
    range[i] = make_int2(first, leafBefore[last] - first + 1);
}

__global__ void fillInt(int32_t* p, int64_t n, int32_t v) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < n) p[i] = v;
}

inline unsigned blocksFor(int64_t n, int t) { return unsigned((n + t - 1) / t); }

}  // namespace

// Device tree construction of the reference topology (treebuild.cu).
cudaError_t gpuBuildTopology(const float* dVerts, int64_t nv, const int32_t* dTris, int64_t nt, int64_t& nLeaves,
                             RefNode*& nodes, int32_t*& irs, int2*& range, bool& closed, Allocator& P, Allocator& A,
                             cudaStream_t s, std::string& err);

// Dipoles and the query layout on the device from the reference nodes in `out.nodes`; `irs` holds
// the internal rank and leaf slot of every node, `range` its leaf-slot range (device arrays).
static cudaError_t finishDeviceTree(const float* dVerts, const int32_t* dTris, const int32_t* irs, const int2* range,
                                    DeviceTree& out, Allocator& P, Allocator& T, cudaStream_t s) {
    const int64_t nNodes = out.nLeaves > 0 ? 2 * out.nLeaves - 1 : 0;
    cudaError_t e;
    int32_t *parent = nullptr, *arrive = nullptr;
    // a refit passes the handle's existing arrays: only missing ones are allocated
    if (!out.faceSlot && (e = P.alloc((void**)&out.faceSlot, sizeof(int32_t) * size_t(std::max<int64_t>(out.nFaces, 1))))) return e;
    fillInt<<<blocksFor(std::max<int64_t>(out.nFaces, 1), 256), 256, 0, s>>>(out.faceSlot, out.nFaces, -1);
    if (nNodes == 0) return cudaGetLastError();
    if (!out.dip8 && (e = P.alloc((void**)&out.dip8, sizeof(float) * 8 * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&parent, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&arrive, sizeof(int32_t) * size_t(nNodes)))) return e;
    const int64_t nInt = std::max<int64_t>(out.nInternal, 1);
    if (!out.cp && (e = P.alloc((void**)&out.cp, sizeof(float4) * 6 * size_t(nInt)))) return e;
    if (!out.dip && (e = P.alloc((void**)&out.dip, sizeof(float4) * 4 * size_t(nInt)))) return e;
    if (!out.tri && (e = P.alloc((void**)&out.tri, sizeof(float4) * 3 * size_t(out.nLeaves)))) return e;
    const unsigned B = blocksFor(nNodes, 256);
    leafDipolesKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, dVerts, dTris, out.dip8, arrive);
    parentsKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, parent);
    sumUpKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, parent, out.dip8, arrive);
    finalizeKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, out.dip8);
    packKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, out.dip8, irs, irs + nNodes, dVerts, dTris, out.cp, out.dip, out.tri,
                                 out.faceSlot);
    obbKernel<<<blocksFor(nNodes, 256), 256, 0, s>>>(nNodes, out.dip8, range, out.tri, parent, irs, irs + nNodes, out.cp);
    // big nodes: chunk counts -> first chunk per node, big-node index -> accumulators
    int32_t *nChunks = nullptr, *chunkStart = nullptr, *isBig = nullptr, *bigIdx = nullptr, *sums = nullptr, *totals = nullptr;
    int* acc = nullptr;
    // a median-split tree has fewer than 2n / kObbChunk nodes above kObbChunk leaves
    const int64_t maxBig = 2 * (out.nLeaves / kObbChunk) + 2;
    if ((e = T.alloc((void**)&nChunks, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&chunkStart, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&isBig, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&bigIdx, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&sums, sizeof(int32_t) * size_t(nNodes / 1024 + 2)))) return e;
    if ((e = T.alloc((void**)&totals, 2 * sizeof(int32_t)))) return e;
    if ((e = T.alloc((void**)&acc, sizeof(int) * 6 * size_t(maxBig)))) return e;
    obbChunkCount<<<B, 256, 0, s>>>(range, nNodes, nChunks, isBig);
    if ((e = exclusiveScanI32(nChunks, chunkStart, nNodes, sums, totals, s))) return e;
    if ((e = exclusiveScanI32(isBig, bigIdx, nNodes, sums, totals + 1, s))) return e;
    obbAccInit<<<blocksFor(6 * maxBig, 256), 256, 0, s>>>(acc, totals + 1, maxBig);
    obbChunkKernel<<<unsigned(numSMs()) * 8, 256, 0, s>>>(nNodes, out.dip8, range, out.tri, chunkStart, totals, bigIdx, maxBig,
                                                           acc, parent);
    obbBigKernel<<<B, 256, 0, s>>>(nNodes, out.dip8, isBig, bigIdx, maxBig, acc, parent, irs, irs + nNodes, out.cp);
    return cudaGetLastError();
}

// Query-tree pointers and the root data that travel in the kernels' parameter block.
static cudaError_t setQueryRoot(DeviceTree& out, cudaStream_t s) {
    cudaError_t e;
    const int64_t nLeaves = out.nLeaves;
    QueryTree& q = out.q;
    q.cp = out.cp;
    q.dip = out.dip;
    q.tri = out.tri;
    q.faceSlot = out.faceSlot;
    q.nodes = reinterpret_cast<const float4*>(out.nodes);
    q.nLeaves = int32_t(out.nLeaves);
    q.nFaces = int32_t(out.nFaces);
    q.closed = out.closed ? 1 : 0;
    if (nLeaves > 0) {  // root data for the kernels' parameter block
        float rd[8];
        RefNode r;
        if ((e = cudaMemcpyAsync(rd, out.dip8, sizeof(rd), cudaMemcpyDeviceToHost, s))) return e;
        if ((e = cudaMemcpyAsync(&r, out.nodes, sizeof(r), cudaMemcpyDeviceToHost, s))) return e;
        if ((e = cudaStreamSynchronize(s))) return e;
        const int32_t rootLink = r.r >= 0 ? 0 : ~0;
        float lf;
        std::memcpy(&lf, &rootLink, 4);
        q.rootDip0 = make_float4(rd[0], rd[1], rd[2], rd[7]);
        q.rootDip1 = make_float4(rd[4], rd[5], rd[6], lf);
        q.rootBox0 = make_float4(r.minx, r.miny, r.minz, lf);
        q.rootBox1 = make_float4(r.maxx, r.maxy, r.maxz, 0.f);
    }
    return cudaStreamSynchronize(s);
}

cudaError_t buildDeviceTree(const float* dVerts, int64_t nv, const int32_t* dTris, int64_t nt, DeviceTree& out,
                            Allocator& P, Allocator& T, cudaStream_t s, std::string& err) {
    cudaError_t e;
    int64_t nLeaves = 0;
    int32_t* irs = nullptr;
    int2* range = nullptr;
    if ((e = gpuBuildTopology(dVerts, nv, dTris, nt, nLeaves, out.nodes, irs, range, out.closed, P, T, s, err))) return e;
    out.nFaces = nt;
    out.nLeaves = nLeaves;
    out.nInternal = nLeaves > 0 ? nLeaves - 1 : 0;
    if ((e = finishDeviceTree(dVerts, dTris, irs, range, out, P, T, s))) return e;
    return setQueryRoot(out, s);
}

cudaError_t refitDeviceTree(const float* dVerts, int64_t nv, const int32_t* dTris, const uint64_t* dChanged, DeviceTree& out,
                            Allocator& P, Allocator& T, cudaStream_t s) {
    const int64_t nNodes = out.nLeaves > 0 ? 2 * out.nLeaves - 1 : 0;
    if (nNodes == 0) return cudaSuccess;
    cudaError_t e;
    int32_t *parent = nullptr, *arrive = nullptr, *flag = nullptr, *before = nullptr, *sums = nullptr, *total = nullptr,
            *irs = nullptr;
    int2* range = nullptr;
    if ((e = T.alloc((void**)&parent, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&arrive, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&flag, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&before, sizeof(int32_t) * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&sums, sizeof(int32_t) * size_t(nNodes / 1024 + 2)))) return e;
    if ((e = T.alloc((void**)&total, sizeof(int32_t)))) return e;
    if ((e = T.alloc((void**)&irs, sizeof(int32_t) * 2 * size_t(nNodes)))) return e;
    if ((e = T.alloc((void**)&range, sizeof(int2) * size_t(nNodes)))) return e;
    const unsigned B = blocksFor(nNodes, 256);
    parentsKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, parent);
    refitLeafKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, dVerts, dTris, dChanged, nv, arrive);
    refitUpKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, parent, arrive);
    leafFlagKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, flag);
    if ((e = exclusiveScanI32(flag, before, nNodes, sums, total, s))) return e;
    ranksKernel<<<B, 256, 0, s>>>(out.nodes, nNodes, before, irs, range);
    if ((e = cudaGetLastError())) return e;
    if ((e = finishDeviceTree(dVerts, dTris, irs, range, out, P, T, s))) return e;
    return setQueryRoot(out, s);
}

}  // namespace gbfwn
