// GPU construction of the reference AABB tree, node for node.
//
// The reference (MRMesh/MRAABBTreeMaker.hpp:51-165, MRMesh/MRAABBTree.cpp:15-60) splits the leaves
// of a node at the median of a total order: box-centre coordinate (min + max) along the node box's
// largest, then middle, then smallest dimension (MRMesh/MRBox.h:376-396, ties of extents broken by
// dimension index), then face id; the floor(n/2) smallest go left, and nodes are stored in
// pre-order (left child = parent + 1, right child = parent + 2 * nLeft).  Because the order is
// total, the split sets depend only on the sets, never on how a partition is computed -- so a
// level-synchronous GPU build reproduces the reference tree exactly:
//
//  * large segments (> kSmall leaves, the top ~10 levels): one level at a time over all segments;
//    node box = segmented min/max reduction; the median is found by an MSB-first radix select on
//    the 128-bit key (three order-preserving coordinate words, then the id), 8 bits per pass,
//    starting below the leading bytes the node box already fixes and stopping as soon as the
//    selected prefix is unique in every segment (the host reads that count every 4 passes; passes
//    after the last needed one return at once); then a stable partition by "key below the median"
//    built on a global exclusive scan;
//  * small segments (2..kSmall leaves): one thread block per segment finishes the whole subtree in
//    shared memory, level by level, ranking every element within its sub-segment by counting.
//
// Leaves come out in pre-order slot order (their final positions), so every node also gets its
// leaf-slot range and its internal-node rank, which the query layout needs.
// Compiled with -fmad=false (no contraction in the box / key arithmetic).
#include <algorithm>
#include <cfloat>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace gbfwn {

namespace {

constexpr int kSmall = 512;  // segments of at most this many leaves are finished in shared memory
constexpr int kScanBlock = 1024;

struct Elem {  // one leaf during construction (40 bytes)
    int32_t id;
    float c[3];   // box min + max per dimension (the comparison key)
    float mn[3], mx[3];
};

// The comparison key of the large-segment levels, kept beside the elements in the same order (one
// 16-byte load, so the radix passes do not stream the 40-byte elements): c[3], then the id.
struct __align__(16) Key {
    float c[3];
    int32_t id;
};

__device__ __forceinline__ uint32_t orderedBits(float f) {
    uint32_t b = __float_as_uint(f == 0.f ? 0.f : f);  // -0 and +0 compare equal in the reference
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// 128-bit key of an element under dims (d2 most significant): w[0] is the most significant word.
__device__ __forceinline__ void keyWords(const Key& e, int d2, int d1, int d0, uint32_t w[4]) {
    w[0] = orderedBits(e.c[d2]);
    w[1] = orderedBits(e.c[d1]);
    w[2] = orderedBits(e.c[d0]);
    w[3] = uint32_t(e.id) ^ 0x80000000u;
}

__device__ __forceinline__ Key loadKey(const Key* k, int32_t p) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(k) + p);
    Key r;
    r.c[0] = v.x;
    r.c[1] = v.y;
    r.c[2] = v.z;
    r.id = __float_as_int(v.w);
    return r;
}

__device__ __forceinline__ int keyByte(const uint32_t w[4], int b) {  // b = 0 is the most significant byte
    return (w[b >> 2] >> (8 * (3 - (b & 3)))) & 0xff;
}

// -1 / 0 / +1 comparing the top `nb` bytes of w against the prefix p
__device__ __forceinline__ int cmpPrefix(const uint32_t w[4], const uint32_t p[4], int nb) {
    for (int i = 0; i < 4; ++i) {
        const int bits = min(32, max(0, 8 * nb - 32 * i));
        if (bits == 0) break;
        const uint32_t mask = bits == 32 ? 0xffffffffu : ~(0xffffffffu >> bits);
        const uint32_t a = w[i] & mask, b = p[i] & mask;
        if (a != b) return a < b ? -1 : 1;
    }
    return 0;
}

__device__ __forceinline__ int floatToOrderedInt(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float orderedIntToFloat(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// MRMesh/MRBox.h:376-396 with the reference's std::pair<float,int> comparison
__device__ __forceinline__ void sortedDims(const float ext[3], int& d0, int& d1, int& d2) {
    float e[3] = {ext[0], ext[1], ext[2]};
    int id[3] = {0, 1, 2};
    for (int i = 0; i + 1 < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (e[j] < e[i] || (e[j] == e[i] && id[j] < id[i])) {
                const float t = e[i];
                e[i] = e[j];
                e[j] = t;
                const int u = id[i];
                id[i] = id[j];
                id[j] = u;
            }
    d0 = id[0];
    d1 = id[1];
    d2 = id[2];
}

struct Seg {
    int32_t root, first, num, large;  // large: 1 if handled by the level path
};

struct SegState {  // radix-select state of a large segment
    uint32_t prefix[4];
    int32_t k;       // rank still to find inside the current prefix bucket
    int32_t nbytes;  // bytes of prefix fixed so far
    int32_t done;
    int32_t dims;    // d0 | d1 << 2 | d2 << 4
};

// ---------------------------------------------------------------- scan (exclusive, int32)
__global__ void scanBlocks(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n, int32_t* __restrict__ sums) {
    __shared__ int32_t warpSums[32];
    const int64_t base = int64_t(blockIdx.x) * kScanBlock;
    const int t = threadIdx.x;  // 256 threads x 4 elements
    int32_t v[4], tot = 0;
    for (int j = 0; j < 4; ++j) {
        const int64_t i = base + 4 * t + j;
        v[j] = i < n ? in[i] : 0;
        tot += v[j];
    }
    int32_t x = tot;
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if ((t & 31) >= o) x += y;
    }
    if ((t & 31) == 31) warpSums[t >> 5] = x;
    __syncthreads();
    if (t < 32) {
        int32_t w = t < 8 ? warpSums[t] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (t >= o) w += y;
        }
        if (t < 8) warpSums[t] = w;
    }
    __syncthreads();
    int32_t excl = x - tot + ((t >> 5) ? warpSums[(t >> 5) - 1] : 0);
    for (int j = 0; j < 4; ++j) {
        const int64_t i = base + 4 * t + j;
        if (i < n) out[i] = excl;
        excl += v[j];
    }
    if (t == 255) sums[blockIdx.x] = excl;
}

__global__ void scanSums(int32_t* sums, int64_t nb, int32_t* total) {  // one block, sequential chunks
    __shared__ int32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nb; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const int32_t v = i < nb ? sums[i] : 0;
        int32_t x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        __shared__ int32_t ws[32];
        if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            int32_t w = ws[threadIdx.x];
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= o) w += y;
            }
            ws[threadIdx.x] = w;
        }
        __syncthreads();
        const int32_t incl = x + ((threadIdx.x >> 5) ? ws[(threadIdx.x >> 5) - 1] : 0);
        if (i < nb) sums[i] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void scanAdd(int32_t* out, int64_t n, const int32_t* sums) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i < n) out[i] += sums[i / kScanBlock];
}

// ---------------------------------------------------------------- leaves
// 64-bit mixing function (the splitmix64 finalizer of Steele, Lea and Flood, 2014).
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// H(a, b) - H(b, a) for the directed edge a -> b under the hash with the given seed.
__device__ __forceinline__ uint64_t edgeTerm(uint32_t a, uint32_t b, uint64_t seed) {
    return mix64(((uint64_t(a) << 32) | b) + seed) - mix64(((uint64_t(b) << 32) | a) + seed);
}

// Valid-face flags and the closedness fingerprint of the valid faces: the sum over their directed
// edges a -> b of H(a, b) - H(b, a), for two seeded 64-bit hashes H.  An undirected edge {a, b}
// contributes (n(a->b) - n(b->a)) (H(a, b) - H(b, a)), so both sums are zero when every edge is
// used as often in each direction -- the faces form a closed oriented surface (a 2-cycle: possibly
// non-manifold or self-intersecting), whose exact winding number is an integer constant on each
// connected region of space off the surface -- and are both zero by chance for an open surface
// with probability about 2^-128.
__global__ void validFaces(const int32_t* __restrict__ tris, int64_t nt, int64_t nv, int32_t* __restrict__ flag,
                           int32_t* __restrict__ err, unsigned long long* __restrict__ fingerprint) {
    const int64_t f = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    uint64_t s0 = 0, s1 = 0;
    if (f < nt) {
        const int32_t a = tris[3 * f], b = tris[3 * f + 1], c = tris[3 * f + 2];
        const bool valid = a >= 0 && b >= 0 && c >= 0;
        if (a >= nv || b >= nv || c >= nv) atomicOr(err, 1);
        flag[f] = valid ? 1 : 0;
        if (valid) {
            constexpr uint64_t k0 = 0x9e3779b97f4a7c15ull, k1 = 0xd1b54a32d192ed03ull;
            s0 = edgeTerm(a, b, k0) + edgeTerm(b, c, k0) + edgeTerm(c, a, k0);
            s1 = edgeTerm(a, b, k1) + edgeTerm(b, c, k1) + edgeTerm(c, a, k1);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
    }
    if ((threadIdx.x & 31) == 0 && (s0 | s1)) {
        atomicAdd(fingerprint, (unsigned long long)s0);
        atomicAdd(fingerprint + 1, (unsigned long long)s1);
    }
}

// MRMesh/MRAABBTree.cpp:15-29: box of the three vertices, then one ulp outwards (MRBox.h:260-270)
__global__ void makeLeaves(const float* __restrict__ verts, const int32_t* __restrict__ tris, int64_t nt,
                           const int32_t* __restrict__ flag, const int32_t* __restrict__ pos, Elem* __restrict__ out,
                           Key* __restrict__ keys) {
    const int64_t f = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (f >= nt || !flag[f]) return;
    Elem e;
    e.id = int32_t(f);
    for (int d = 0; d < 3; ++d) {
        float lo = FLT_MAX, hi = -FLT_MAX;
        for (int k = 0; k < 3; ++k) {
            const float x = verts[3 * int64_t(tris[3 * f + k]) + d];
            if (x < lo) lo = x;
            if (x > hi) hi = x;
        }
        e.mn[d] = nextafterf(lo, -FLT_MAX);
        e.mx[d] = nextafterf(hi, FLT_MAX);
        e.c[d] = e.mn[d] + e.mx[d];
    }
    out[pos[f]] = e;
    keys[pos[f]] = Key{{e.c[0], e.c[1], e.c[2]}, e.id};
}

__device__ __forceinline__ void writeLeaf(const Elem& e, int32_t node, int32_t slot, RefNode* nodes, int32_t* irs, int2* range,
                                          int64_t nNodes) {
    nodes[node] = RefNode{e.mn[0], e.mn[1], e.mn[2], e.mx[0], e.mx[1], e.mx[2], e.id, -1};
    irs[node] = -1;
    irs[nNodes + node] = slot;
    range[node] = make_int2(slot, 1);
}

__device__ __forceinline__ void writeInternal(const float mn[3], const float mx[3], int32_t root, int32_t first, int32_t num,
                                              RefNode* nodes, int32_t* irs, int2* range, int64_t nNodes) {
    const int32_t nl = num / 2;
    nodes[root] = RefNode{mn[0], mn[1], mn[2], mx[0], mx[1], mx[2], root + 1, root + 2 * nl};
    irs[root] = root - first;  // internal nodes before it = pre-order index - leaves before it
    irs[nNodes + root] = -1;
    range[root] = make_int2(first, num);
}

// ---------------------------------------------------------------- large-segment level
// Every element carries its entry in the current level's segment list (segOf, -1 when its segment
// is not split on this path), so the per-element kernels below need no search.

__global__ void __launch_bounds__(256) segBoxes(const Elem* __restrict__ el, int32_t n, const int32_t* __restrict__ segOf,
                                                int* __restrict__ box) {
    __shared__ int sSeg[8];
    __shared__ float sV[8][6];
    const int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int s = -1;
    Elem e;
    if (p < n) {
        s = segOf[p];
        if (s >= 0) e = el[p];
    }
    const unsigned same = __match_any_sync(0xffffffffu, s);
    float v[6] = {FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX, FLT_MAX};
    if (s >= 0) {  // all as minima
        v[0] = e.mn[0]; v[1] = e.mn[1]; v[2] = e.mn[2];
        v[3] = -e.mx[0]; v[4] = -e.mx[1]; v[5] = -e.mx[2];
    }
    const int leader = __ffs(same) - 1;
    if (same == 0xffffffffu) {  // the whole warp in one segment (the common case): butterfly
        for (int j = 0; j < 6; ++j)
            for (int off = 16; off; off >>= 1) v[j] = fminf(v[j], __shfl_xor_sync(0xffffffffu, v[j], off));
    } else {
        for (int j = 0; j < 6; ++j) {  // reduce inside the group of lanes of the same segment
            unsigned m = same;
            float r = FLT_MAX;
            while (m) {
                const int src = __ffs(m) - 1;
                r = fminf(r, __shfl_sync(same, v[j], src));
                m &= m - 1;
            }
            v[j] = r;
        }
    }
    // a block whose 256 elements all lie in one segment (most blocks of the upper levels) reduces its
    // eight warps in shared memory and updates the segment box once instead of eight times
    if (lane == 0) sSeg[w] = same == 0xffffffffu ? s : -1;
    __syncthreads();
    bool uniform = sSeg[0] >= 0;
    for (int k = 1; k < 8; ++k) uniform = uniform && sSeg[k] == sSeg[0];
    if (uniform) {
        if (lane == 0)
            for (int j = 0; j < 6; ++j) sV[w][j] = v[j];
        __syncthreads();
        if (threadIdx.x < 6) {
            const int j = threadIdx.x;
            float r = sV[0][j];
            for (int k = 1; k < 8; ++k) r = fminf(r, sV[k][j]);
            if (j < 3) atomicMin(&box[6 * s + j], floatToOrderedInt(r));
            else atomicMax(&box[6 * s + j], floatToOrderedInt(-r));
        }
        return;
    }
    if (s >= 0 && lane == leader) {
        for (int j = 0; j < 3; ++j) atomicMin(&box[6 * s + j], floatToOrderedInt(v[j]));
        for (int j = 0; j < 3; ++j) atomicMax(&box[6 * s + 3 + j], floatToOrderedInt(-v[3 + j]));
    }
}

__global__ void segInit(const Seg* __restrict__ segs, int nseg, int* __restrict__ box, SegState* __restrict__ st, int* hist) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    for (int j = 0; j < 3; ++j) {
        box[6 * s + j] = floatToOrderedInt(FLT_MAX);
        box[6 * s + 3 + j] = floatToOrderedInt(-FLT_MAX);
    }
    SegState z;
    for (int j = 0; j < 4; ++j) z.prefix[j] = 0;
    z.k = segs[s].num / 2;
    z.nbytes = 0;
    z.done = segs[s].large ? 0 : 1;
    z.dims = 0;
    st[s] = z;
}

__global__ void segNodes(const Seg* __restrict__ segs, int nseg, const int* __restrict__ box, SegState* __restrict__ st,
                         RefNode* nodes, int32_t* irs, int2* range, int64_t nNodes) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg || !segs[s].large) return;
    float mn[3], mx[3], ext[3];
    for (int j = 0; j < 3; ++j) {
        mn[j] = orderedIntToFloat(box[6 * s + j]);
        mx[j] = orderedIntToFloat(box[6 * s + 3 + j]);
        ext[j] = mx[j] - mn[j];
    }
    int d0, d1, d2;
    sortedDims(ext, d0, d1, d2);
    st[s].dims = d0 | (d1 << 2) | (d2 << 4);
    // every leaf's key word c[d2] = mn + mx lies in [min mn + min mn, max mx + max mx] (rounding is
    // monotone), so the leading bytes both ends share are the median's too: the select starts below them
    const uint32_t lo = orderedBits(mn[d2] + mn[d2]), hi = orderedBits(mx[d2] + mx[d2]);
    const int nb = (lo ^ hi) ? (__clz(lo ^ hi) >> 3) : 4;
    st[s].prefix[0] = nb == 4 ? lo : (nb == 0 ? 0u : lo & ~(0xffffffffu >> (8 * nb)));
    st[s].nbytes = nb;
    writeInternal(mn, mx, segs[s].root, segs[s].first, segs[s].num, nodes, irs, range, nNodes);
}

__global__ void radixHist(const Key* __restrict__ keys, int32_t n, const int32_t* __restrict__ segOf,
                          const SegState* __restrict__ st, int* __restrict__ hist, const int* __restrict__ prevPending) {
    if (prevPending && *prevPending == 0) return;  // every segment finished in an earlier pass
    const int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    const int s = p < n ? segOf[p] : -1;
    if (s >= 0) {
        const SegState S = st[s];
        if (!S.done) {
            uint32_t w[4];
            keyWords(loadKey(keys, p), (S.dims >> 4) & 3, (S.dims >> 2) & 3, S.dims & 3, w);
            if (cmpPrefix(w, S.prefix, S.nbytes) == 0) key = 256 * s + keyByte(w, S.nbytes);
        }
    }
    const unsigned grp = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && (threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&hist[key], __popc(grp));
}

// one warp per segment: pick the bucket holding rank k, extend the prefix, clear the histogram
__global__ void radixSelect(const Seg* __restrict__ segs, int nseg, SegState* __restrict__ st, int* __restrict__ hist,
                            int* __restrict__ pending, const int* __restrict__ prevPending) {
    if (prevPending && *prevPending == 0) return;
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= nseg) return;
    SegState S = st[s];
    if (S.done) return;
    int cnt[8], sum = 0;
    for (int j = 0; j < 8; ++j) {
        cnt[j] = hist[256 * s + 8 * lane + j];
        sum += cnt[j];
    }
    int incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const int excl = incl - sum;
    int bucket = -1, before = 0, bcount = 0;
    if (S.k >= excl && S.k < incl) {
        int c = excl;
        for (int j = 0; j < 8; ++j) {
            if (S.k < c + cnt[j]) {
                bucket = 8 * lane + j;
                before = c;
                bcount = cnt[j];
                break;
            }
            c += cnt[j];
        }
    }
    const unsigned who = __ballot_sync(0xffffffffu, bucket >= 0);
    if (who == 0) {  // cannot happen (k < bucket total by construction); stop this segment safely
        for (int j = 0; j < 8; ++j) hist[256 * s + 8 * lane + j] = 0;
        if (lane == 0) st[s].done = 1;
        return;
    }
    const int src = __ffs(who) - 1;
    bucket = __shfl_sync(0xffffffffu, bucket, src);
    before = __shfl_sync(0xffffffffu, before, src);
    bcount = __shfl_sync(0xffffffffu, bcount, src);
    for (int j = 0; j < 8; ++j) hist[256 * s + 8 * lane + j] = 0;
    if (lane == 0) {
        const int b = S.nbytes;
        S.prefix[b >> 2] |= uint32_t(bucket) << (8 * (3 - (b & 3)));
        S.nbytes = b + 1;
        S.k -= before;
        if (bcount <= 1 || S.nbytes == 16) S.done = 1;
        else atomicAdd(pending, 1);
        st[s] = S;
    }
}

__global__ void partFlags(const Key* __restrict__ keys, int32_t n, const int32_t* __restrict__ segOf,
                          const SegState* __restrict__ st, int32_t* __restrict__ flag) {
    const int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int s = segOf[p];
    int f = 0;
    if (s >= 0) {
        const SegState S = st[s];
        uint32_t w[4];
        keyWords(loadKey(keys, p), (S.dims >> 4) & 3, (S.dims >> 2) & 3, S.dims & 3, w);
        f = cmpPrefix(w, S.prefix, S.nbytes) < 0 ? 1 : 0;  // strictly below the median element: left
    }
    flag[p] = f;
}

// also writes the element's segment at the next level: child c of segment s is entry 2s + c of the
// next segment list, or -1 when that child is finished elsewhere (kSmall leaves or fewer)
__global__ void partScatter(const Elem* __restrict__ el, Elem* __restrict__ out, const Key* __restrict__ keys,
                            Key* __restrict__ keysOut, int32_t n, const Seg* __restrict__ segs,
                            const int32_t* __restrict__ segOf, int32_t* __restrict__ segOfNext,
                            const int32_t* __restrict__ flag, const int32_t* __restrict__ scan) {
    const int32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int s = segOf[p];
    int32_t dst = p, next = -1;
    if (s >= 0) {
        const int32_t first = segs[s].first, num = segs[s].num, k = num / 2;
        const int32_t leftBefore = scan[p] - scan[first];
        const bool left = flag[p] != 0;
        dst = left ? first + leftBefore : first + k + ((p - first) - leftBefore);
        if ((left ? k : num - k) > kSmall) next = 2 * s + (left ? 0 : 1);
    }
    out[dst] = el[p];
    reinterpret_cast<float4*>(keysOut)[dst] = __ldg(reinterpret_cast<const float4*>(keys) + p);
    segOfNext[dst] = next;
}

// children of every large segment; small ones are queued for the shared-memory finish, single
// leaves written at once
__global__ void segChildren(const Seg* __restrict__ segs, int nseg, Seg* __restrict__ next, const Elem* __restrict__ el,
                            Seg* __restrict__ small, int* __restrict__ nsmall, RefNode* nodes, int32_t* irs, int2* range,
                            int64_t nNodes) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const Seg S = segs[s];
    if (!S.large) {  // keeps the slot so segments stay sorted by first; no longer processed
        next[2 * s] = Seg{S.root, S.first, S.num, 0};
        next[2 * s + 1] = Seg{S.root, S.first + S.num, 0, 0};
        return;
    }
    const int32_t k = S.num / 2;
    const Seg L{S.root + 1, S.first, k, 0}, R{S.root + 2 * k, S.first + k, S.num - k, 0};
    const Seg ch[2] = {L, R};
    for (int c = 0; c < 2; ++c) {
        Seg C = ch[c];
        if (C.num > kSmall) {
            C.large = 1;
        } else if (C.num >= 2) {
            small[atomicAdd(nsmall, 1)] = C;
        } else if (C.num == 1) {
            writeLeaf(el[C.first], C.root, C.first, nodes, irs, range, nNodes);
        }
        next[2 * s + c] = C;
    }
}

// ---------------------------------------------------------------- small segments
struct SubSeg {
    int16_t first, num;
    int32_t root;
    int32_t dims;
    int32_t bmin[3], bmax[3];
};

// two element buffers, the sub-segments of two levels, each element's sort key for the current level
// (16 bytes, 16-byte aligned after the elements), its sub-segment, the sub-segment counts
constexpr size_t kFinishSmem =
    sizeof(Elem) * 2 * kSmall + sizeof(float4) * kSmall + sizeof(SubSeg) * kSmall + sizeof(int16_t) * kSmall + 16;

__global__ void __launch_bounds__(kSmall) finishSmall(const Elem* __restrict__ el, const Seg* __restrict__ small,
                                                   RefNode* nodes, int32_t* irs, int2* range, int64_t nNodes) {
    extern __shared__ __align__(16) unsigned char smem[];
    Elem(*buf)[kSmall] = reinterpret_cast<Elem(*)[kSmall]>(smem);
    float4* key = reinterpret_cast<float4*>(smem + sizeof(Elem) * 2 * kSmall);
    unsigned char* rest = smem + sizeof(Elem) * 2 * kSmall + sizeof(float4) * kSmall;
    SubSeg(*sub)[kSmall / 2] = reinterpret_cast<SubSeg(*)[kSmall / 2]>(rest);
    int16_t* sid = reinterpret_cast<int16_t*>(rest + sizeof(SubSeg) * kSmall);
    int* nsub = reinterpret_cast<int*>(rest + sizeof(SubSeg) * kSmall + sizeof(int16_t) * kSmall);
    const Seg S = small[blockIdx.x];
    const int t = threadIdx.x;
    for (int i = t; i < S.num; i += blockDim.x) {
        buf[0][i] = el[S.first + i];
        sid[i] = -1;
    }
    if (t == 0) {
        sub[0][0] = SubSeg{0, int16_t(S.num), S.root, 0, {0, 0, 0}, {0, 0, 0}};
        nsub[0] = 1;
    }
    __syncthreads();
    int cur = 0;
    while (nsub[cur] > 0) {
        const int ns = nsub[cur];
        // element -> sub-segment map, box init
        for (int j = t; j < ns; j += blockDim.x) {
            const SubSeg& q = sub[cur][j];
            for (int i = q.first; i < q.first + q.num; ++i) sid[i] = int16_t(j);
            for (int d = 0; d < 3; ++d) {
                sub[cur][j].bmin[d] = floatToOrderedInt(FLT_MAX);
                sub[cur][j].bmax[d] = floatToOrderedInt(-FLT_MAX);
            }
        }
        __syncthreads();
        for (int i = t; i < S.num; i += blockDim.x) {
            const int j = sid[i];
            if (j < 0) continue;
            const Elem& e = buf[cur][i];
            for (int d = 0; d < 3; ++d) {
                atomicMin(&sub[cur][j].bmin[d], floatToOrderedInt(e.mn[d]));
                atomicMax(&sub[cur][j].bmax[d], floatToOrderedInt(e.mx[d]));
            }
        }
        __syncthreads();
        for (int j = t; j < ns; j += blockDim.x) {
            SubSeg& q = sub[cur][j];
            float mn[3], mx[3], ext[3];
            for (int d = 0; d < 3; ++d) {
                mn[d] = orderedIntToFloat(q.bmin[d]);
                mx[d] = orderedIntToFloat(q.bmax[d]);
                ext[d] = mx[d] - mn[d];
            }
            int d0, d1, d2;
            sortedDims(ext, d0, d1, d2);
            q.dims = d0 | (d1 << 2) | (d2 << 4);
            writeInternal(mn, mx, q.root, S.first + q.first, q.num, nodes, irs, range, nNodes);
        }
        __syncthreads();
        // each element's key in its sub-segment's order: (c[d2], c[d1], c[d0], id), one 16-byte load
        for (int i = t; i < S.num; i += blockDim.x) {
            const int j = sid[i];
            if (j < 0) continue;
            const int dims = sub[cur][j].dims;
            const Elem& e = buf[cur][i];
            key[i] = make_float4(e.c[(dims >> 4) & 3], e.c[(dims >> 2) & 3], e.c[dims & 3], __int_as_float(e.id));
        }
        __syncthreads();
        // rank of every element inside its sub-segment = its position after the split
        for (int i = t; i < S.num; i += blockDim.x) {
            const int j = sid[i];
            if (j < 0) {
                buf[cur ^ 1][i] = buf[cur][i];
                continue;
            }
            const SubSeg q = sub[cur][j];
            const float4 me = key[i];
            const int myId = __float_as_int(me.w);
            int rank = 0;
            for (int o = q.first; o < q.first + q.num; ++o) {
                const float4 f = key[o];
                const bool less = f.x != me.x   ? f.x < me.x
                                  : f.y != me.y ? f.y < me.y
                                  : f.z != me.z ? f.z < me.z
                                                : __float_as_int(f.w) < myId;
                rank += less ? 1 : 0;
            }
            buf[cur ^ 1][q.first + rank] = buf[cur][i];
        }
        __syncthreads();
        if (t == 0) nsub[cur ^ 1] = 0;
        __syncthreads();
        for (int j = t; j < ns; j += blockDim.x) {
            const SubSeg q = sub[cur][j];
            const int k = q.num / 2;
            const SubSeg ch[2] = {SubSeg{q.first, int16_t(k), q.root + 1, 0, {0, 0, 0}, {0, 0, 0}},
                                  SubSeg{int16_t(q.first + k), int16_t(q.num - k), q.root + 2 * k, 0, {0, 0, 0}, {0, 0, 0}}};
            for (int c = 0; c < 2; ++c) {
                if (ch[c].num >= 2) sub[cur ^ 1][atomicAdd(&nsub[cur ^ 1], 1)] = ch[c];
                else writeLeaf(buf[cur ^ 1][ch[c].first], ch[c].root, S.first + ch[c].first, nodes, irs, range, nNodes);
            }
        }
        for (int i = t; i < S.num; i += blockDim.x) sid[i] = -1;
        __syncthreads();
        cur ^= 1;
    }
}

inline unsigned blocks(int64_t n, int t) { return unsigned((n + t - 1) / t); }

}  // namespace

cudaError_t exclusiveScanI32(const int32_t* in, int32_t* out, int64_t n, int32_t* sums, int32_t* total, cudaStream_t s) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (n == 0) return cudaMemsetAsync(total, 0, sizeof(int32_t), s);
    scanBlocks<<<unsigned(nb), 256, 0, s>>>(in, out, n, sums);
    scanSums<<<1, 1024, 0, s>>>(sums, nb, total);
    scanAdd<<<blocks(n, 256), 256, 0, s>>>(out, n, sums);
    return cudaGetLastError();
}

namespace {
cudaError_t exclusiveScan(const int32_t* in, int32_t* out, int64_t n, int32_t* sums, int32_t* total, cudaStream_t s) {
    return exclusiveScanI32(in, out, n, sums, total, s);
}
}  // namespace

// Builds the reference tree on the device.  Outputs: nodes (2n-1 reference nodes, allocated through
// P), irs (2 x (2n-1): internal rank, leaf slot) and range (first slot, count), allocated through the
// temporary allocator A like every other work array.  nLeaves = number
// of valid faces.  Returns cudaErrorInvalidValue with `err` set when a vertex id is out of range.
cudaError_t gpuBuildTopology(const float* dVerts, int64_t nv, const int32_t* dTris, int64_t nt, int64_t& nLeaves,
                             RefNode*& nodes, int32_t*& irs, int2*& range, bool& closed, Allocator& P, Allocator& A,
                             cudaStream_t s, std::string& err) {
    cudaError_t e;
    nLeaves = 0;
    closed = false;
    nodes = nullptr;
    irs = nullptr;
    range = nullptr;
    if (nt == 0) return cudaSuccess;
    int32_t *flag = nullptr, *pos = nullptr, *sums = nullptr, *misc = nullptr;
    const int64_t nbMax = (nt + kScanBlock - 1) / kScanBlock + 1;
    if ((e = A.alloc((void**)&flag, sizeof(int32_t) * size_t(nt)))) return e;
    if ((e = A.alloc((void**)&pos, sizeof(int32_t) * size_t(nt)))) return e;
    if ((e = A.alloc((void**)&sums, sizeof(int32_t) * size_t(nbMax)))) return e;
    // [0] error, [1] total, [3] nsmall, [4..7] closedness fingerprint (2 x u64), [16..31] pending per pass
    if ((e = A.alloc((void**)&misc, sizeof(int32_t) * 32))) return e;
    int32_t* pend = misc + 16;
    if ((e = cudaMemsetAsync(misc, 0, sizeof(int32_t) * 8, s))) return e;
    validFaces<<<blocks(nt, 256), 256, 0, s>>>(dTris, nt, nv, flag, misc, reinterpret_cast<unsigned long long*>(misc + 4));
    if ((e = exclusiveScan(flag, pos, nt, sums, misc + 1, s))) return e;
    int32_t hm[8];
    if ((e = cudaMemcpyAsync(hm, misc, sizeof(hm), cudaMemcpyDeviceToHost, s))) return e;
    if ((e = cudaStreamSynchronize(s))) return e;
    if (hm[0]) {
        err = "triangle vertex id out of range";
        return cudaErrorInvalidValue;
    }
    closed = (hm[4] | hm[5] | hm[6] | hm[7]) == 0;
    const int32_t n = hm[1];
    nLeaves = n;
    if (n == 0) return cudaSuccess;
    const int64_t nNodes = 2 * int64_t(n) - 1;
    Elem *el = nullptr, *el2 = nullptr;
    Key *keys = nullptr, *keys2 = nullptr;
    if ((e = A.alloc((void**)&el, sizeof(Elem) * size_t(n)))) return e;
    if ((e = A.alloc((void**)&el2, sizeof(Elem) * size_t(n)))) return e;
    if ((e = A.alloc((void**)&keys, sizeof(Key) * size_t(n)))) return e;
    if ((e = A.alloc((void**)&keys2, sizeof(Key) * size_t(n)))) return e;
    if ((e = P.alloc((void**)&nodes, sizeof(RefNode) * size_t(nNodes)))) return e;
    if ((e = A.alloc((void**)&irs, sizeof(int32_t) * 2 * size_t(nNodes)))) return e;
    if ((e = A.alloc((void**)&range, sizeof(int2) * size_t(nNodes)))) return e;
    makeLeaves<<<blocks(nt, 256), 256, 0, s>>>(dVerts, dTris, nt, flag, pos, el, keys);
    // segment lists: at most 2^L entries at level L; the large-segment levels stop below n / kSmall
    int maxSegs = 1;
    while (maxSegs < 2 * (n / kSmall + 1)) maxSegs <<= 1;
    maxSegs *= 2;
    Seg *segA = nullptr, *segB = nullptr, *small = nullptr;
    SegState* st = nullptr;
    int* box = nullptr;
    int* hist = nullptr;
    const int64_t maxSmall = 2 * (int64_t(n) / 2 + 1);
    if ((e = A.alloc((void**)&segA, sizeof(Seg) * size_t(maxSegs)))) return e;
    if ((e = A.alloc((void**)&segB, sizeof(Seg) * size_t(maxSegs)))) return e;
    if ((e = A.alloc((void**)&small, sizeof(Seg) * size_t(maxSmall)))) return e;
    if ((e = A.alloc((void**)&st, sizeof(SegState) * size_t(maxSegs)))) return e;
    if ((e = A.alloc((void**)&box, sizeof(int) * 6 * size_t(maxSegs)))) return e;
    if ((e = A.alloc((void**)&hist, sizeof(int) * 256 * size_t(maxSegs)))) return e;
    int32_t* scan = pos;  // reuse: n <= nt
    int32_t *segOf = nullptr, *segOf2 = nullptr;  // each element's entry in the current segment list, -1 if none
    if ((e = A.alloc((void**)&segOf, sizeof(int32_t) * size_t(n)))) return e;
    if ((e = A.alloc((void**)&segOf2, sizeof(int32_t) * size_t(n)))) return e;
    int nsmallHost = 0;
    const Seg root{0, 0, n, n > kSmall ? 1 : 0};
    if (n > kSmall) {
        if ((e = cudaMemcpyAsync(segA, &root, sizeof(Seg), cudaMemcpyHostToDevice, s))) return e;
        if ((e = cudaMemsetAsync(segOf, 0, sizeof(int32_t) * size_t(n), s))) return e;
        // histogram rows are cleared once here; every select pass clears the rows it read, so they
        // are zero again at the start of each level
        if ((e = cudaMemsetAsync(hist, 0, sizeof(int) * 256 * size_t(maxSegs), s))) return e;
        int nseg = 1;
        for (int level = 0; level < 40; ++level) {
            segInit<<<blocks(nseg, 128), 128, 0, s>>>(segA, nseg, box, st, hist);
            segBoxes<<<blocks(n, 256), 256, 0, s>>>(el, n, segOf, box);
            segNodes<<<blocks(nseg, 128), 128, 0, s>>>(segA, nseg, box, st, nodes, irs, range, nNodes);
            // pass p counts its unfinished segments in pend[p]; a pass after one that left none returns
            // at once, so the host reads the count only every kGroup passes
            constexpr int kGroup = 4;
            if ((e = cudaMemsetAsync(pend, 0, sizeof(int32_t) * 16, s))) return e;
            for (int pass = 0; pass < 16; ++pass) {
                const int* prev = pass ? pend + pass - 1 : nullptr;
                radixHist<<<blocks(n, 256), 256, 0, s>>>(keys, n, segOf, st, hist, prev);
                radixSelect<<<blocks(int64_t(nseg) * 32, 256), 256, 0, s>>>(segA, nseg, st, hist, pend + pass, prev);
                if ((pass + 1) % kGroup && pass != 15) continue;
                int32_t pending = 0;
                if ((e = cudaMemcpyAsync(&pending, pend + pass, sizeof(int32_t), cudaMemcpyDeviceToHost, s))) return e;
                if ((e = cudaStreamSynchronize(s))) return e;
                if (pending == 0) break;
            }
            partFlags<<<blocks(n, 256), 256, 0, s>>>(keys, n, segOf, st, flag);
            if ((e = exclusiveScan(flag, scan, n, sums, misc + 1, s))) return e;
            partScatter<<<blocks(n, 256), 256, 0, s>>>(el, el2, keys, keys2, n, segA, segOf, segOf2, flag, scan);
            std::swap(el, el2);
            std::swap(keys, keys2);
            std::swap(segOf, segOf2);
            segChildren<<<blocks(nseg, 128), 128, 0, s>>>(segA, nseg, segB, el, small, misc + 3, nodes, irs, range, nNodes);
            std::swap(segA, segB);
            nseg *= 2;
            // any large segment left?  (the largest child has ceil(num/2) leaves)
            int64_t largest = n;
            for (int l = 0; l <= level; ++l) largest = (largest + 1) / 2;
            if (largest <= kSmall || nseg > maxSegs / 2) break;
        }
        if ((e = cudaMemcpyAsync(&nsmallHost, misc + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, s))) return e;
        if ((e = cudaStreamSynchronize(s))) return e;
    } else if (n >= 2) {
        if ((e = cudaMemcpyAsync(small, &root, sizeof(Seg), cudaMemcpyHostToDevice, s))) return e;
        nsmallHost = 1;
    }
    if (n == 1) {  // a single leaf is the whole tree
        Elem h;
        if ((e = cudaMemcpyAsync(&h, el, sizeof(Elem), cudaMemcpyDeviceToHost, s))) return e;
        if ((e = cudaStreamSynchronize(s))) return e;
        const RefNode leaf{h.mn[0], h.mn[1], h.mn[2], h.mx[0], h.mx[1], h.mx[2], h.id, -1};
        const int32_t hirs[2] = {-1, 0};
        const int2 hr = make_int2(0, 1);
        if ((e = cudaMemcpyAsync(nodes, &leaf, sizeof(leaf), cudaMemcpyHostToDevice, s))) return e;
        if ((e = cudaMemcpyAsync(irs, hirs, sizeof(hirs), cudaMemcpyHostToDevice, s))) return e;
        if ((e = cudaMemcpyAsync(range, &hr, sizeof(hr), cudaMemcpyHostToDevice, s))) return e;
        return cudaStreamSynchronize(s);
    }
    if (nsmallHost > 0) {
        if ((e = cudaFuncSetAttribute(finishSmall, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kFinishSmem)))) return e;
        finishSmall<<<unsigned(nsmallHost), kSmall, kFinishSmem, s>>>(el, small, nodes, irs, range, nNodes);
    }
    return cudaGetLastError();
}

}  // namespace gbfwn
