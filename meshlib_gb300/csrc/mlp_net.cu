// Surrogate signed-distance network: Fourier features -> 4 x (128, SiLU) -> 1, BF16 weights and
// activations on the tensor cores with FP32 accumulation (training: the GEMMs of mlp_gemm.cu;
// inference: the fused inferKernel below), trained on the GPU on
// samples whose signed distances come from the exact traversal, then used to cull 8x8x8-voxel
// bricks that lie outside a requested distance band.
//
// Network (74,369 parameters): u = (p - centre) * scale (the grid box mapped to [-1, 1]^3);
// features f[64 a + 2 k] = sin(w_k u_a), f[64 a + 2 k + 1] = cos(w_k u_a), w_k = pi * 2^(k / 5),
// k < 32, a < 3 (192 features); h1 = silu(W1 f + b1), h_l = silu(W_l h_{l-1} + b_l) for l = 2..4;
// y = w5 . h4 + b5.  Target: the signed distance clamped to +-clampD; loss = mean squared error.
#include <cuda_bf16.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "common.cuh"
#include "handle.cuh"
#include "mlp.cuh"
#include "surrogate.cuh"
#include "mlp_tiles.cuh"
#include "umma.cuh"

namespace gbfwn {

namespace {

constexpr int kF = kMlpF, kH = kMlpH, kFreq = kMlpFreq;
static_assert(kOffB5 + 1 == kSurrogateParams, "parameter layout");

inline unsigned nblk(int64_t n, int t) { return unsigned((n + t - 1) / t); }

// ---------------------------------------------------------------- random numbers (hash based)
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float urand(uint32_t seed, uint32_t i, uint32_t k) {
    return (hash32(seed * 0x9e3779b9u ^ hash32(i * 4u + k)) >> 8) * (1.f / 16777216.f);
}

// ---------------------------------------------------------------- Adam + weight packing
// Cosine learning-rate schedule from lr0 to lr0/100 over `total` steps; the step counter lives on
// the device so that a captured step can be replayed.
__global__ void adamKernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                           int n, const int32_t* __restrict__ stepPtr, int total, float lr0, float b1, float b2, float eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int step = *stepPtr + 1;
    const float frac = fminf(1.f, float(step) / float(max(total, 1)));
    const float lr = lr0 * (0.01f + 0.99f * 0.5f * (1.f + cospif(frac)));
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.f - powf(b1, float(step)));
    const float vh = vi / (1.f - powf(b2, float(step)));
    p[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void stepCounterKernel(int32_t* step, int32_t* off, int batch, int batchesPerEpoch) {
    const int s = *step + 1;
    *step = s;
    *off = (s % batchesPerEpoch) * batch;
}

// bf16 copies of W1..W4 as the shared-memory images the fused training step and inference copy in
// (mlp.cuh: 128-row x 64-column K-major blocks with the 128-byte swizzle)
__device__ __forceinline__ int64_t imageIndex(int block, int r, int c) {  // element (r, c) of a 64-column block
    return int64_t(block) * (kImgBlockBytes / 2) + r * 64 + (((c >> 3) ^ (r & 7)) << 3) + (c & 7);
}
__global__ void packKernel(const float* __restrict__ params, __nv_bfloat16* __restrict__ img) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kH * kF) {
        const int r = i / kF, c = i % kF;
        img[imageIndex(c / 64, r, c % 64)] = __float2bfloat16(params[kOffW1 + i]);
    }
    if (i < 3 * kH * kH) {
        const int l = i / (kH * kH), r = (i / kH) % kH, c = i % kH;
        const int off = (l == 0 ? kOffW2 : l == 1 ? kOffW3 : kOffW4);
        img[imageIndex(3 + 2 * l + c / 64, r, c % 64)] = __float2bfloat16(params[off + r * kH + c]);
    }
}

// ---------------------------------------------------------------- sampling
// Uniform samples: a jittered lattice over the box, consecutive samples neighbours (4x4x2 blocks of
// lattice cells) so that the exact traversal's warp packets stay coherent.
__global__ void uniformSamplesKernel(float* __restrict__ pts, int n, int m, float3 lo, float3 cell, uint32_t seed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int blk = i >> 5, ln = i & 31;
    const int bx = (m + 3) / 4, by = (m + 3) / 4;
    const int cx = (blk % bx) * 4 + (ln & 3), cy = ((blk / bx) % by) * 4 + ((ln >> 2) & 3), cz = (blk / (bx * by)) * 2 + (ln >> 4);
    pts[3 * int64_t(i) + 0] = lo.x + (float(cx % m) + urand(seed, i, 0)) * cell.x;
    pts[3 * int64_t(i) + 1] = lo.y + (float(cy % m) + urand(seed, i, 1)) * cell.y;
    pts[3 * int64_t(i) + 2] = lo.z + (float(cz % m) + urand(seed, i, 2)) * cell.z;
}

// Near-surface samples: leaf slots in order (spatially coherent), a uniform point of the triangle,
// offset along its normal by a normal deviate of standard deviation sigma.
__global__ void surfaceSamplesKernel(float* __restrict__ pts, int n, const float4* __restrict__ tri, int nLeaves, float sigma,
                                     float3 lo, float3 hi, uint32_t seed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || nLeaves == 0) return;
    const int slot = int((int64_t(i) * nLeaves) / n);
    const float4 A = tri[3 * int64_t(slot)], B = tri[3 * int64_t(slot) + 1], C = tri[3 * int64_t(slot) + 2];
    float r1 = urand(seed, i, 0), r2 = urand(seed, i, 1);
    if (r1 + r2 > 1.f) {
        r1 = 1.f - r1;
        r2 = 1.f - r2;
    }
    const float3 ab = make_float3(B.x - A.x, B.y - A.y, B.z - A.z), ac = make_float3(C.x - A.x, C.y - A.y, C.z - A.z);
    float3 nrm = make_float3(ab.y * ac.z - ab.z * ac.y, ab.z * ac.x - ab.x * ac.z, ab.x * ac.y - ab.y * ac.x);
    const float nl = sqrtf(nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z);
    if (nl > 0.f) {
        nrm.x /= nl;
        nrm.y /= nl;
        nrm.z /= nl;
    }
    // Box-Muller
    const float u1 = fmaxf(urand(seed, i, 2), 1e-7f), u2 = urand(seed, i, 3);
    const float off = sigma * sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
    // kept inside the box the network serves (it is never evaluated outside it)
    pts[3 * int64_t(i) + 0] = fminf(fmaxf(A.x + r1 * ab.x + r2 * ac.x + off * nrm.x, lo.x), hi.x);
    pts[3 * int64_t(i) + 1] = fminf(fmaxf(A.y + r1 * ab.y + r2 * ac.y + off * nrm.y, lo.y), hi.y);
    pts[3 * int64_t(i) + 2] = fminf(fmaxf(A.z + r1 * ab.z + r2 * ac.z + off * nrm.z, lo.z), hi.z);
}

__global__ void absErrMaxKernel(const float* __restrict__ pred, const float* __restrict__ target, int n, float clampD,
                                unsigned* __restrict__ maxBits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.f;
    if (i < n) e = fabsf(pred[i] - fminf(fmaxf(target[i], -clampD), clampD));
    for (int o = 16; o; o >>= 1) e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxBits, __float_as_uint(e));  // e >= 0: bits are ordered
}

// largest overstatement of the distance, |pred| - |d|, over samples with |d| < limit
__global__ void overestimateMaxKernel(const float* __restrict__ pred, const float* __restrict__ target, int n, float limit,
                                      unsigned* __restrict__ maxBits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.f;
    if (i < n) {
        const float d = fabsf(target[i]);
        if (d < limit) e = fmaxf(fabsf(pred[i]) - d, 0.f);
    }
    for (int o = 16; o; o >>= 1) e = fmaxf(e, __shfl_xor_sync(0xffffffffu, e, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxBits, __float_as_uint(e));
}

// ---------------------------------------------------------------- bricks
__global__ void brickCentersKernel(float* __restrict__ pts, int3 bdims, int3 dims, Xf xf) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bdims.x * bdims.y * bdims.z) return;
    const int bx = b % bdims.x, by = (b / bdims.x) % bdims.y, bz = b / (bdims.x * bdims.y);
    // centre of the voxels the brick actually holds (edge bricks are partial)
    const float cx = 0.5f * float(8 * bx + min(8 * bx + 7, dims.x - 1));
    const float cy = 0.5f * float(8 * by + min(8 * by + 7, dims.y - 1));
    const float cz = 0.5f * float(8 * bz + min(8 * bz + 7, dims.z - 1));
    pts[3 * b + 0] = xf.a[0] * cx + xf.a[1] * cy + xf.a[2] * cz + xf.b[0];
    pts[3 * b + 1] = xf.a[3] * cx + xf.a[4] * cy + xf.a[5] * cz + xf.b[1];
    pts[3 * b + 2] = xf.a[6] * cx + xf.a[7] * cy + xf.a[8] * cz + xf.b[2];
}

// keep[b] = 1 unless every voxel of brick b is certainly at distance >= band:
// |d(v)| >= |d(c)| - |v - c| >= lowerBound(c) - radius.
__global__ void brickKeepKernel(const float* __restrict__ lowerBound, int nb, float band, float radius, int32_t* __restrict__ keep) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const float lb = lowerBound[b];
    keep[b] = (lb - radius >= band) ? 0 : 1;
}

// Runs of kept bricks stacked in z, at most kRunBricks long: a run starts at a kept brick whose brick
// below is not kept, or at every kRunBricks-th brick layer.  A run's tile columns carry their seeds
// and signs from brick to brick.  512^3, band 0.01 diag, exact pass over the 30,016 kept bricks:
// 1 brick per run 10.06 ms, 2 9.83 ms, 4 9.77 ms, unlimited 14.2 ms (the runs down the sides of the
// shape are long and leave the tail to a few warps).
constexpr int kRunBricks = 2;
__global__ void runStartKernel(const int32_t* __restrict__ keep, int3 bd, int32_t* __restrict__ start) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int nb = bd.x * bd.y * bd.z;
    if (b >= nb) return;
    const int layer = bd.x * bd.y;
    start[b] = (keep[b] && (b < layer || !keep[b - layer] || (b / layer) % kRunBricks == 0)) ? 1 : 0;
}

// (bx, by, bz0, count) of every run, in the order of their first bricks
__global__ void runKernel(const int32_t* __restrict__ keep, const int32_t* __restrict__ start, const int32_t* __restrict__ pos,
                          int3 bd, int4* __restrict__ runs) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int nb = bd.x * bd.y * bd.z;
    if (b >= nb || !start[b]) return;
    const int layer = bd.x * bd.y;
    const int bx = b % bd.x, by = (b / bd.x) % bd.y, bz = b / layer;
    int n = 1;
    while (bz + n < bd.z && (bz + n) % kRunBricks != 0 && keep[b + n * layer]) ++n;
    runs[pos[b]] = make_int4(bx, by, bz, n);
}

// NaN everywhere (voxels of culled bricks stay NaN); 16-byte stores when p is 16-byte aligned
__global__ void fillNanKernel(float* __restrict__ p, int64_t n) {
    const float nan = __int_as_float(0x7fc00000);
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    const int64_t i0 = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
    if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
        float4* p4 = reinterpret_cast<float4*>(p);
        for (int64_t i = i0; i < n / 4; i += stride) p4[i] = make_float4(nan, nan, nan, nan);
        for (int64_t i = 4 * (n / 4) + i0; i < n; i += stride) p[i] = nan;
    } else {
        for (int64_t i = i0; i < n; i += stride) p[i] = nan;
    }
}

// lower bound of |d| at each brick centre from the surrogate: |pred| - margin
__global__ void surrogateLowerBound(const float* __restrict__ pred, int n, float margin, float* __restrict__ lb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) lb[i] = fabsf(pred[i]) - margin;
}

// lower bound from the exact unsigned distance computed with maxDistSq = (band + radius)^2: NaN
// (not finite) means the distance is at least band + radius, so the brick is out whatever the
// rounding of (band + radius) - radius (+inf, not band + radius)
__global__ void exactLowerBound(const float* __restrict__ d, int n, float* __restrict__ lb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) lb[i] = isfinite(d[i]) ? fabsf(d[i]) : INFINITY;
}

// ---------------------------------------------------------------- fused inference
// The whole network for 128 points per step in one persistent CTA per SM (512 threads): the bf16
// weight images (W1 as three 64-wide K blocks, W2..W4 as two: 144 KB, already in the 128-byte swizzle)
// arrive once by TMA bulk copy; per tile the threads write the Fourier features straight into the
// swizzled activation tile (axis a = K block a), one thread issues the layer's tcgen05 MMAs
// (M = N = 128, K = 16 each) into a 128-column TMEM accumulator and commits them to an mbarrier, and
// the epilogue (warp w: TMEM lanes 32 (w % 4).., columns 32 (w / 4)..) adds the bias, applies SiLU,
// rounds to bf16 and writes the next layer's input tile in place -- the activations never leave the
// SM.  Rounding points and SiLU arithmetic are the training step's (features, h1..h4 in bf16; FP32
// accumulation); the output layer sums bf16(h4) * w5 in FP32.  A timed-out wait sets status bit 1.
constexpr int kInferThreads = 512;
constexpr int kInferParts = kInferThreads / 128;  // threads per row
constexpr int kTileBytes = 128 * 128;  // one 128-row x 64-column bf16 K block
constexpr size_t kInferSmem = 1024 + size_t(kTileBytes) * (kImgBlocks + 3);

__global__ void __launch_bounds__(kInferThreads, 1) inferKernel(const float* __restrict__ pts, int n, NetMeta meta,
                                                                 const __nv_bfloat16* __restrict__ img,
                                                                 const float* __restrict__ params, float* __restrict__ out,
                                                                 unsigned* status) {
    extern __shared__ __align__(1024) uint8_t smemRaw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
    uint8_t* wt = smem;                             // 9 weight blocks: W1 0..2, W2 3..4, W3 5..6, W4 7..8
    uint8_t* at = smem + kImgBlocks * kTileBytes;   // 3 activation blocks
    __shared__ __align__(8) uint64_t bar, barW;
    __shared__ uint32_t tmemBase;
    __shared__ float partial[kInferParts][128];
    __shared__ int failed;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    if (warp == 0) umma::tmemAlloc(&tmemBase, 128);
    if (t == 0) {
        umma::mbarInit(&bar, 1);
        umma::mbarInit(&barW, 1);
        failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        umma::bulkLoad(wt, img, uint32_t(kImgBlocks) * kTileBytes, &barW);
    }
    umma::fenceBeforeSync();
    __syncthreads();
    umma::fenceAfterSync();
    const uint32_t tmem = tmemBase;
    constexpr uint32_t idesc = umma::idescBf16(128, 128);
    const int q = warp & 3, part = warp >> 2;  // TMEM lane quarter, column part
    const int erow = 32 * q + lane;            // this thread's row in the epilogue
    const int cb = 32 * part;                  // its first column
    const uint32_t tq = tmem + (uint32_t(32 * q) << 16);
    const float b5 = params[kOffB5];
    uint32_t phase = 0;
    bool weightsIn = false;  // the weight copy's barrier has completed (thread 0)
    const int numTiles = (n + 127) / 128;
    for (int tile = blockIdx.x; tile < numTiles; tile += gridDim.x) {
        // features: thread (row, part) writes frequencies 8 part .. 8 part + 7 of every axis
        {
            constexpr int kChunks = 8 / kInferParts;
            const int row = t & 127, fh = t >> 7;
            const int64_t i = int64_t(tile) * 128 + row;
            const bool live = i < n;
            float u[3] = {0.f, 0.f, 0.f};
            if (live)
                for (int a = 0; a < 3; ++a) u[a] = (pts[3 * i + a] - meta.center[a]) * meta.scale;
            for (int a = 0; a < 3; ++a)
                for (int c = kChunks * fh; c < kChunks * fh + kChunks; ++c) {  // chunk c = frequencies 4c .. 4c + 3
                    uint32_t w[4];
                    for (int j = 0; j < 4; ++j) {
                        float sv = 0.f, cv = 0.f;
                        if (live) sincosf(meta.freq[4 * c + j] * u[a], &sv, &cv);
                        w[j] = mlp::packBf16x2(sv, cv);
                    }
                    *reinterpret_cast<uint4*>(at + a * kTileBytes + row * 128 + ((c ^ (row & 7)) << 4)) =
                        make_uint4(w[0], w[1], w[2], w[3]);
                }
        }
        for (int layer = 0; layer < 4; ++layer) {
            umma::fenceProxyAsync();
            umma::fenceBeforeSync();
            __syncthreads();
            if (t == 0) {
                umma::fenceAfterSync();
                if (!weightsIn) {
                    weightsIn = umma::mbarWait(&barW, 0);
                    if (!weightsIn) atomicOr(&failed, 1);
                }
                const int nk = layer == 0 ? 3 : 2;
                const uint8_t* wb = wt + (layer == 0 ? 0 : 3 + 2 * (layer - 1)) * kTileBytes;
                for (int b = 0; b < nk; ++b) {
                    const uint32_t sa = umma::smemAddr(at + b * kTileBytes), sb = umma::smemAddr(wb + b * kTileBytes);
                    for (int kk = 0; kk < 4; ++kk)
                        umma::mmaBf16(tmem, umma::descK128(sa + 32 * kk), umma::descK128(sb + 32 * kk), idesc,
                                      (b > 0 || kk > 0) ? 1u : 0u);
                }
                umma::commit(&bar);
            }
            if (!umma::mbarWait(&bar, phase)) atomicOr(&failed, 1);
            phase ^= 1u;
            __syncthreads();
            if (failed) break;
            umma::fenceAfterSync();
            const float* bias = params + (layer == 0 ? kOffB1 : layer == 1 ? kOffB2 : layer == 2 ? kOffB3 : kOffB4);
            float v[32];
            umma::tmemLoad32(tq + uint32_t(cb), v);
            float acc5 = 0.f;
            for (int h = 0; h < 2; ++h) {
                float b[16];
                mlp::loadParams16(bias + cb + 16 * h, b);
                uint32_t w[8];
                for (int j = 0; j < 16; j += 2) w[j / 2] = mlp::packBf16x2(mlp::silu(v[16 * h + j] + b[j]), mlp::silu(v[16 * h + j + 1] + b[j + 1]));
                if (layer < 3) {
                    mlp::storeRow16(at, erow, cb + 16 * h, w);  // next layer's input, in place
                } else {
                    float w5[16];
                    mlp::loadParams16(params + kOffW5 + cb + 16 * h, w5);
                    for (int j = 0; j < 16; j += 2) {
                        const __nv_bfloat162 hb = *reinterpret_cast<const __nv_bfloat162*>(&w[j / 2]);
                        acc5 += __low2float(hb) * w5[j] + __high2float(hb) * w5[j + 1];
                    }
                }
            }
            if (layer == 3) partial[part][erow] = acc5;
        }
        if (failed) break;
        __syncthreads();
        if (t < 128) {
            const int64_t i = int64_t(tile) * 128 + t;
            float y = b5;
            for (int p2 = 0; p2 < kInferParts; ++p2) y += partial[p2][t];
            if (i < n) out[i] = y;
        }
    }
    if (t == 0 && !weightsIn) {  // no tile, or a timed-out wait: the weight copy must land before the CTA exits
        if (!umma::mbarWait(&barW, 0)) atomicOr(&failed, 1);
    }
    if (failed && t == 0 && status) atomicOr(status, 2u);
    umma::fenceBeforeSync();
    __syncthreads();
    if (warp == 0) umma::tmemFree(tmem, 128);
}

}  // namespace

// ------------------------------------------------------------------------------------------------
struct SurrogateNet::Work {
    int batch = 0;
    __nv_bfloat16* spill = nullptr;  // 32 KB per 128-row tile of a training step
};

SurrogateNet::~SurrogateNet() { release(); }

int SurrogateNet::workRows() const { return work_ ? work_->batch : 0; }

void SurrogateNet::release() {
    for (void* p : mem_) cudaFree(p);
    mem_.clear();
    delete work_;
    work_ = nullptr;

    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
}

cudaError_t SurrogateNet::alloc(void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (!e) mem_.push_back(*p);
    return e;
}

cudaError_t SurrogateNet::init(uint64_t seed) {
    cudaError_t e;
    if ((e = prepareTrainStep())) return e;
    if ((e = cudaFuncSetAttribute(inferKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kInferSmem)))) return e;
    if ((e = alloc((void**)&params_, sizeof(float) * kSurrogateParams))) return e;
    if ((e = alloc((void**)&grads_, sizeof(float) * kSurrogateParams))) return e;
    if ((e = alloc((void**)&m_, sizeof(float) * kSurrogateParams))) return e;
    if ((e = alloc((void**)&v_, sizeof(float) * kSurrogateParams))) return e;
    if ((e = alloc((void**)&img_, size_t(kImgBlockBytes) * kImgBlocks))) return e;
    if ((e = alloc((void**)&counters_, sizeof(int32_t) * 4))) return e;
    if ((e = alloc((void**)&scalars_, sizeof(float) * 8))) return e;
    for (int k = 0; k < kFreq; ++k) meta.freq[k] = float(M_PI * std::pow(2.0, k / 5.0));
    // He-uniform hidden layers, small output layer, zero biases (deterministic from the seed)
    std::vector<float> h(kSurrogateParams, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fanOut, int fanIn, float gain) {
        const float lim = gain * std::sqrt(3.f / float(fanIn));
        std::uniform_real_distribution<float> U(-lim, lim);
        for (int i = 0; i < fanOut * fanIn; ++i) h[off + i] = U(rng);
    };
    fill(kOffW1, kH, kF, 1.0f);
    fill(kOffW2, kH, kH, 1.4142f);
    fill(kOffW3, kH, kH, 1.4142f);
    fill(kOffW4, kH, kH, 1.4142f);
    fill(kOffW5, 1, kH, 0.1f);
    return setParams(h.data(), nullptr);
}

cudaError_t SurrogateNet::setParams(const float* hostParams, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(params_, hostParams, sizeof(float) * kSurrogateParams, cudaMemcpyHostToDevice, s);
    if (!e) e = cudaMemsetAsync(m_, 0, sizeof(float) * kSurrogateParams, s);
    if (!e) e = cudaMemsetAsync(v_, 0, sizeof(float) * kSurrogateParams, s);
    if (!e) e = cudaMemsetAsync(counters_, 0, sizeof(int32_t) * 4, s);
    if (e) return e;
    return pack(s);
}

cudaError_t SurrogateNet::getParams(float* hostParams, cudaStream_t s) const {
    cudaError_t e = cudaMemcpyAsync(hostParams, params_, sizeof(float) * kSurrogateParams, cudaMemcpyDeviceToHost, s);
    return e ? e : cudaStreamSynchronize(s);
}

cudaError_t SurrogateNet::pack(cudaStream_t s) {
    packKernel<<<nblk(3 * kH * kH, 256), 256, 0, s>>>(params_, img_);
    return cudaGetLastError();
}

cudaError_t SurrogateNet::ensureWork(int batchPad) {
    if (work_) return cudaSuccess;  // sized once per network; inference walks larger inputs in chunks
    work_ = new Work;
    work_->batch = batchPad;
    return alloc((void**)&work_->spill, size_t(kImgBlockBytes) * 2 * size_t((batchPad + 127) / 128));
}

// One training (or gradient-only) step over `n` rows taken from pts/targets through idx (or the
// first n rows when idx is null), padded to nPad rows: the fused forward + backward kernel
// (mlp_train.cu), then Adam, the bf16 repacking and the batch offset.  Leaves the loss in scalars_[0].
cudaError_t SurrogateNet::step(const float* pts, const float* targets, const int32_t* idx, int64_t idxMod, int n, int nPad,
                               bool update, int totalSteps, float lr, cudaStream_t s) {
    if (!work_ || nPad > work_->batch) return cudaErrorInvalidValue;
    cudaError_t e;
    if ((e = cudaMemsetAsync(grads_, 0, sizeof(float) * kSurrogateParams, s))) return e;
    if ((e = cudaMemsetAsync(scalars_, 0, sizeof(float), s))) return e;
    TrainStepArgs a;
    a.pts = pts;
    a.targets = targets;
    a.idx = idx;
    a.offPtr = idx ? counters_ + 1 : nullptr;
    a.idxMod = idxMod;
    a.n = n;
    a.nPad = nPad;
    a.clampD = meta.clampD;
    a.params = params_;
    a.img = img_;
    a.spill = work_->spill;
    a.grads = grads_;
    a.loss = scalars_;
    a.status = reinterpret_cast<unsigned*>(counters_ + 3);
    if ((e = launchTrainStep(a, meta, s))) return e;
    if (!update) return cudaGetLastError();
    adamKernel<<<nblk(kSurrogateParams, 256), 256, 0, s>>>(params_, grads_, m_, v_, kSurrogateParams, counters_, totalSteps, lr,
                                                          0.9f, 0.99f, 1e-8f);
    if ((e = pack(s))) return e;
    stepCounterKernel<<<1, 1, 0, s>>>(counters_, counters_ + 1, nPad, int(idxMod / nPad));
    return cudaGetLastError();
}

cudaError_t SurrogateNet::infer(const float* pts, int64_t n, float* out, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (n > int64_t(INT32_MAX) - 128) return cudaErrorInvalidValue;
    const int tiles = int((n + 127) / 128);
    const int grid = std::max(1, std::min(tiles, numSMs()));
    inferKernel<<<grid, kInferThreads, kInferSmem, s>>>(pts, int(n), meta, img_, params_, out,
                                                        reinterpret_cast<unsigned*>(counters_ + 3));
    return cudaGetLastError();
}

cudaError_t SurrogateNet::train(const QueryTree& t, unsigned* scratch, const TrainOptions& o, TrainStats& st, cudaStream_t s) {
    cudaError_t e;
    const auto t0 = std::chrono::steady_clock::now();
    const int batch = (o.batch + 127) / 128 * 128;
    int64_t nTrain = std::max<int64_t>(o.samples / batch, 1) * batch;
    if ((e = ensureWork(batch))) return e;
    float *pts = nullptr, *dist = nullptr;
    int32_t* idx = nullptr;
    const int64_t nAll = nTrain + o.validation;
    if ((e = alloc((void**)&pts, sizeof(float) * 3 * size_t(nAll)))) return e;
    if ((e = alloc((void**)&dist, sizeof(float) * size_t(nAll)))) return e;
    if ((e = alloc((void**)&idx, sizeof(int32_t) * size_t(nTrain)))) return e;
    // samples: half uniform in the box, half near the surface; the validation set likewise
    auto gen = [&](float* p, int64_t n, uint32_t seed) -> cudaError_t {
        const int64_t nu = n / 2, ns = n - nu;
        const int m = std::max(1, int(std::ceil(std::cbrt(double(nu)))));
        const float3 cell = make_float3((o.hi[0] - o.lo[0]) / m, (o.hi[1] - o.lo[1]) / m, (o.hi[2] - o.lo[2]) / m);
        if (nu) uniformSamplesKernel<<<nblk(nu, 256), 256, 0, s>>>(p, int(nu), m, make_float3(o.lo[0], o.lo[1], o.lo[2]), cell, seed);
        if (ns)
            surfaceSamplesKernel<<<nblk(ns, 256), 256, 0, s>>>(p + 3 * nu, int(ns), t.tri, t.nLeaves, o.sigma,
                                                               make_float3(o.lo[0], o.lo[1], o.lo[2]),
                                                               make_float3(o.hi[0], o.hi[1], o.hi[2]), seed ^ 0x5bd1e995u);
        return cudaGetLastError();
    };
    if ((e = gen(pts, nTrain, uint32_t(o.seed)))) return e;
    if (o.validation && (e = gen(pts + 3 * nTrain, o.validation, uint32_t(o.seed * 31 + 7)))) return e;
    const DistOpts exact{0.f, 3.402823466e+38f, 0, 0.5f, o.beta};
    if ((e = launchVectorSdf(t, pts, nAll, exact, 1, dist, scratch, s))) return e;
    // batches are slices of a random permutation of the training samples
    {
        std::vector<int32_t> perm(static_cast<size_t>(nTrain));
        for (int64_t i = 0; i < nTrain; ++i) perm[i] = int32_t(i);
        std::mt19937_64 rng(o.seed * 2654435761ull + 1);
        std::shuffle(perm.begin(), perm.end(), rng);
        if ((e = cudaMemcpyAsync(idx, perm.data(), sizeof(int32_t) * perm.size(), cudaMemcpyHostToDevice, s))) return e;
        if ((e = cudaStreamSynchronize(s))) return e;
    }
    const auto t1 = std::chrono::steady_clock::now();
    // capture one optimizer step in a CUDA graph and replay it
    cudaStream_t cs;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking))) return e;
    cudaGraph_t g = nullptr;
    if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal))) return e;
    e = step(pts, dist, idx, nTrain, batch, batch, true, o.steps, o.lr, cs);
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    if (e || e2) {
        if (g) cudaGraphDestroy(g);
        cudaStreamDestroy(cs);
        return e ? e : e2;
    }
    if (graph_) cudaGraphExecDestroy(graph_);
    e = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e) return e;
    std::vector<float> lossHist;
    for (int it = 0; it < o.steps; ++it) {
        if ((e = cudaGraphLaunch(graph_, s))) return e;
        if ((it + 1) % 500 == 0 || it + 1 == o.steps) {
            float l = 0.f;
            if ((e = cudaMemcpyAsync(&l, scalars_, sizeof(float), cudaMemcpyDeviceToHost, s))) return e;
            if ((e = cudaStreamSynchronize(s))) return e;
            lossHist.push_back(l);
        }
    }
    if ((e = cudaStreamSynchronize(s))) return e;
    const auto t2 = std::chrono::steady_clock::now();
    // validation on held-out samples: the worst error overall (two-sided, against the clamped
    // target) and the worst overstatement of |d| where |d| < limit -> the two margins
    float valMax = 0.f, valOver = 0.f;
    const float limit = o.limit > 0.f ? std::min(o.limit, meta.clampD) : meta.clampD;
    if (o.validation) {
        float* pred = nullptr;
        unsigned* mx = nullptr;
        if ((e = alloc((void**)&pred, sizeof(float) * size_t(o.validation)))) return e;
        if ((e = alloc((void**)&mx, 2 * sizeof(unsigned)))) return e;
        if ((e = infer(pts + 3 * nTrain, o.validation, pred, s))) return e;
        if ((e = cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned), s))) return e;
        absErrMaxKernel<<<nblk(o.validation, 256), 256, 0, s>>>(pred, dist + nTrain, int(o.validation), meta.clampD, mx);
        overestimateMaxKernel<<<nblk(o.validation, 256), 256, 0, s>>>(pred, dist + nTrain, int(o.validation), limit, mx + 1);
        unsigned bits[2] = {0, 0};
        if ((e = cudaMemcpyAsync(bits, mx, sizeof(bits), cudaMemcpyDeviceToHost, s))) return e;
        if ((e = cudaStreamSynchronize(s))) return e;
        std::memcpy(&valMax, &bits[0], 4);
        std::memcpy(&valOver, &bits[1], 4);
    }
    meta.marginAll = o.marginScale * valMax + o.marginFloor;
    meta.margin = o.marginScale * valOver + o.marginFloor;
    meta.limit = limit;
    st.trainLoss = lossHist.empty() ? 0.f : lossHist.back();
    st.valMaxErr = valMax;
    st.valOverestimate = valOver;
    st.limit = limit;
    st.margin = meta.margin;
    st.sampleSeconds = std::chrono::duration<float>(t1 - t0).count();
    st.trainSeconds = std::chrono::duration<float>(t2 - t1).count();
    st.steps = o.steps;
    unsigned status = 0;
    cudaMemcpy(&status, counters_ + 3, sizeof(unsigned), cudaMemcpyDeviceToHost);
    return status ? cudaErrorLaunchTimeout : cudaSuccess;
}

// Banded signed distance: NaN wherever |d| >= band, exact elsewhere.  Bricks of 8x8x8 voxels are
// culled when a lower bound of |d| at their centre minus their half diagonal is >= band; the lower
// bound comes from the surrogate (|pred| - margin) or, with net == null, from the exact unsigned
// distance capped at band + radius.  The kept bricks go through the exact kernel.
cudaError_t bandedGrid(const QueryTree& t, SurrogateNet* net, const GridRange& g, const Xf& xf, const DistOpts& o, int precise,
                       float* out, unsigned* scratch, BandedStats& st, cudaStream_t s) {
    const int3 dims = make_int3(g.nx, g.ny, g.nz);
    const int3 bd = make_int3((g.nx + 7) / 8, (g.ny + 7) / 8, (g.nz + 7) / 8);
    const int nb = bd.x * bd.y * bd.z;
    const float band = std::sqrt(o.maxDistSq);
    // largest distance from a brick's centre to its voxel centres: the image of the corner
    // offsets (+-3.5, +-3.5, +-3.5) voxels under the linear part (edge bricks are smaller)
    float radius = 0.f;
    for (int c = 0; c < 8; ++c) {
        const float d[3] = {(c & 1) ? 3.5f : -3.5f, (c & 2) ? 3.5f : -3.5f, (c & 4) ? 3.5f : -3.5f};
        float r2 = 0.f;
        for (int a = 0; a < 3; ++a) {
            const float w = xf.a[3 * a] * d[0] + xf.a[3 * a + 1] * d[1] + xf.a[3 * a + 2] * d[2];
            r2 += w * w;
        }
        radius = std::fmax(radius, std::sqrt(r2));
    }
    radius *= 1.0001f;
    cudaError_t e;
    float *centers = nullptr, *lb = nullptr, *tmp = nullptr;
    int32_t *keep = nullptr, *pos = nullptr, *start = nullptr, *sums = nullptr, *total = nullptr;
    int4* runs = nullptr;
    std::vector<void*> mem;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaMemPool_t pool = devicePool(dev);  // the library's pool keeps the memory for the next call
    auto A = [&](void** p, size_t b) {
        cudaError_t r = pool ? cudaMallocFromPoolAsync(p, b ? b : 16, pool, s) : cudaMallocAsync(p, b ? b : 16, s);
        if (!r) mem.push_back(*p);
        return r;
    };
    auto done = [&](cudaError_t r) {
        for (void* p : mem) cudaFreeAsync(p, s);
        return r;
    };
    if ((e = A((void**)&centers, sizeof(float) * 3 * size_t(nb)))) return done(e);
    if ((e = A((void**)&lb, sizeof(float) * size_t(nb)))) return done(e);
    if ((e = A((void**)&tmp, sizeof(float) * size_t(nb)))) return done(e);
    if ((e = A((void**)&keep, sizeof(int32_t) * size_t(nb)))) return done(e);
    if ((e = A((void**)&pos, sizeof(int32_t) * size_t(nb)))) return done(e);
    if ((e = A((void**)&start, sizeof(int32_t) * size_t(nb)))) return done(e);
    if ((e = A((void**)&runs, sizeof(int4) * size_t(nb)))) return done(e);
    if ((e = A((void**)&sums, sizeof(int32_t) * size_t(nb / 1024 + 2)))) return done(e);
    if ((e = A((void**)&total, 2 * sizeof(int32_t)))) return done(e);
    // closed mesh, vertical z axis: the signs from the columns' crossings (bits, then crossing lists)
    uint32_t* bits = nullptr;
    void* lists = nullptr;
    const bool columns = signColumnsApply(t, xf, o.beta, o.threshold);
    if (columns) {
        if ((e = A((void**)&bits, signBitsBytes(g)))) return done(e);
        if ((e = A(&lists, signColumnsWorkBytes(g)))) return done(e);
    }
    cudaEvent_t ev[4];
    for (auto& x : ev) cudaEventCreate(&x);
    cudaEventRecord(ev[0], s);
    brickCentersKernel<<<nblk(nb, 256), 256, 0, s>>>(centers, bd, dims, xf);
    if (net) {
        if ((e = net->infer(centers, nb, tmp, s))) return done(e);
        // the one-sided margin is validated for |d| < limit, which covers every brick centre that can
        // hold an in-band voxel (|d(c)| < band + radius) only when band + radius <= limit; otherwise
        // the two-sided margin over all samples applies
        const float m = (band + radius <= net->meta.limit) ? net->meta.margin : std::max(net->meta.margin, net->meta.marginAll);
        surrogateLowerBound<<<nblk(nb, 256), 256, 0, s>>>(tmp, nb, m, lb);
    } else {
        const float cap = band + radius;
        const DistOpts co{0.f, cap * cap, 1, o.threshold, o.beta};
        if ((e = launchVectorSdf(t, centers, nb, co, precise, tmp, scratch, s))) return done(e);
        exactLowerBound<<<nblk(nb, 256), 256, 0, s>>>(tmp, nb, lb);
    }
    brickKeepKernel<<<nblk(nb, 256), 256, 0, s>>>(lb, nb, band, radius, keep);
    if ((e = exclusiveScanI32(keep, pos, nb, sums, total, s))) return done(e);  // the kept count
    runStartKernel<<<nblk(nb, 256), 256, 0, s>>>(keep, bd, start);
    if ((e = exclusiveScanI32(start, pos, nb, sums, total + 1, s))) return done(e);
    runKernel<<<nblk(nb, 256), 256, 0, s>>>(keep, start, pos, bd, runs);
    int32_t counts[2] = {0, 0};  // kept bricks, runs
    if ((e = cudaMemcpyAsync(counts, total, sizeof(counts), cudaMemcpyDeviceToHost, s))) return done(e);
    cudaEventRecord(ev[1], s);
    fillNanKernel<<<unsigned(numSMs()) * 8, 256, 0, s>>>(out, int64_t(g.nx) * g.ny * g.nz);
    if ((e = cudaStreamSynchronize(s))) return done(e);
    cudaEventRecord(ev[2], s);
    const int32_t kept = counts[0];
    if (kept > 0 && columns &&
        (e = launchSignColumns(t, g, xf, o.beta, o.threshold, precise, bits, nullptr, lists, signColumnsWorkBytes(g), scratch, s)))
        return done(e);
    void* fix = nullptr;  // the precise paired walk's fix list
    if (kept > 0 && columns && precise && (e = A(&fix, pairFixBytesForRuns(counts[1], kept)))) return done(e);
    if (kept > 0 && (e = launchGridSdfBricks(t, g, xf, o, precise, out, runs, counts[1], kept, bits, fix, scratch, s))) return done(e);
    cudaEventRecord(ev[3], s);
    if ((e = cudaStreamSynchronize(s))) return done(e);
    cudaEventElapsedTime(&st.cullMs, ev[0], ev[1]);
    cudaEventElapsedTime(&st.exactMs, ev[2], ev[3]);
    for (auto& x : ev) cudaEventDestroy(x);
    st.bricks = nb;
    st.keptBricks = kept;
    return done(cudaGetLastError());
}

}  // namespace gbfwn
