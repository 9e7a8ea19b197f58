// Spatial ordering of arbitrary query points: 30-bit Morton codes (10 bits per axis inside the
// mesh box) sorted by a stable LSD radix sort, 8 bits per pass.  Point queries (calcFromVector,
// distances at points) then walk the points in this order, so the 32 lanes of a warp hold nearby
// points and the packet traversals stay coherent; results are scattered back to the caller's order.
#include <cstdint>

#include "common.cuh"

namespace gbfwn {

namespace {

constexpr int kSortThreads = 256;  // one element per thread, 256 elements per tile

__device__ __forceinline__ uint32_t spread10(uint32_t v) {  // 10 bits -> every third bit
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void mortonKernel(const float* __restrict__ pts, int64_t n, float3 lo, float3 inv, uint32_t* __restrict__ key,
                             int32_t* __restrict__ val) {
    const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const float c[3] = {(pts[3 * i] - lo.x) * inv.x, (pts[3 * i + 1] - lo.y) * inv.y, (pts[3 * i + 2] - lo.z) * inv.z};
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
        const float t = fminf(fmaxf(c[a], 0.f), 1.f) * 1023.f;
        q[a] = uint32_t(t == t ? t : 0.f);  // NaN coordinates sort first
    }
    key[i] = spread10(q[0]) | (spread10(q[1]) << 1) | (spread10(q[2]) << 2);
    val[i] = int32_t(i);
}

// counts[bin * nTiles + tile] = occurrences of digit `bin` in tile
__global__ void histKernel(const uint32_t* __restrict__ key, int64_t n, int shift, int32_t* __restrict__ counts, int nTiles) {
    __shared__ int32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t i = int64_t(blockIdx.x) * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(key[i] >> shift) & 0xff], 1);
    __syncthreads();
    counts[int64_t(threadIdx.x) * nTiles + blockIdx.x] = h[threadIdx.x];
}

// stable scatter: rank inside the tile = elements of lower index with the same digit
__global__ void scatterKernel(const uint32_t* __restrict__ key, const int32_t* __restrict__ val, int64_t n, int shift,
                              const int32_t* __restrict__ offsets, int nTiles, uint32_t* __restrict__ keyOut,
                              int32_t* __restrict__ valOut) {
    __shared__ int32_t warpHist[kSortThreads / 32][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j = threadIdx.x; j < (kSortThreads / 32) * 256; j += kSortThreads) (&warpHist[0][0])[j] = 0;
    __syncthreads();
    const int64_t i = int64_t(blockIdx.x) * kSortThreads + threadIdx.x;
    const bool live = i < n;
    const uint32_t k = live ? key[i] : 0xffffffffu;
    const int digit = live ? int((k >> shift) & 0xff) : 256;  // 256: padding lanes, own group
    const unsigned same = __match_any_sync(0xffffffffu, digit);
    const int rankInWarp = __popc(same & ((1u << lane) - 1u));
    if (live && rankInWarp == 0) warpHist[warp][digit] = __popc(same);
    __syncthreads();
    if (!live) return;
    int before = 0;
    for (int w = 0; w < warp; ++w) before += warpHist[w][digit];
    const int64_t dst = int64_t(offsets[int64_t(digit) * nTiles + blockIdx.x]) + before + rankInWarp;
    keyOut[dst] = k;
    valOut[dst] = val[i];
}

}  // namespace

int64_t mortonOrderScratch(int64_t n) {  // int32 words of scratch mortonOrder needs
    const int64_t tiles = (n + kSortThreads - 1) / kSortThreads;
    const int64_t counts = 256 * tiles;
    return 3 * n + 2 * counts + counts / 1024 + 4;
}

cudaError_t mortonOrder(const float* pts, int64_t n, const float lo[3], const float hi[3], int32_t* order, int32_t* scratch,
                        cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int nTiles = int((n + kSortThreads - 1) / kSortThreads);
    const int64_t nc = int64_t(256) * nTiles;
    uint32_t* keyA = reinterpret_cast<uint32_t*>(scratch);
    uint32_t* keyB = keyA + n;
    int32_t* valB = scratch + 2 * n;
    int32_t* counts = scratch + 3 * n;
    int32_t* offsets = counts + nc;
    int32_t* sums = offsets + nc;
    int32_t* total = sums + nc / 1024 + 2;
    float3 l = make_float3(lo[0], lo[1], lo[2]);
    float3 inv = make_float3(hi[0] > lo[0] ? 1.f / (hi[0] - lo[0]) : 0.f, hi[1] > lo[1] ? 1.f / (hi[1] - lo[1]) : 0.f,
                             hi[2] > lo[2] ? 1.f / (hi[2] - lo[2]) : 0.f);
    mortonKernel<<<unsigned((n + 255) / 256), 256, 0, s>>>(pts, n, l, inv, keyA, order);
    int32_t* valA = order;
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 8 * pass;
        histKernel<<<nTiles, kSortThreads, 0, s>>>(keyA, n, shift, counts, nTiles);
        cudaError_t e = exclusiveScanI32(counts, offsets, nc, sums, total, s);
        if (e) return e;
        scatterKernel<<<nTiles, kSortThreads, 0, s>>>(keyA, valA, n, shift, offsets, nTiles, keyB, valB);
        std::swap(keyA, keyB);
        std::swap(valA, valB);
    }
    // four passes: the sorted indices are back in `order`
    return cudaGetLastError();
}

}  // namespace gbfwn
