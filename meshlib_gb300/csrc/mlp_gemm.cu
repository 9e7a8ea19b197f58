// BF16 GEMM on the 5th-generation tensor cores (tcgen05), FP32 accumulation in TMEM, with the
// epilogues the surrogate network needs.  D[M x N] = A[M x K] * B[N x K]^T, A and B both K-major
// (row-major with K contiguous), M a multiple of 128, N in {128, 192}, K a multiple of 64.
//
// One CTA (4 warps) computes a 128-row tile over the full N: K is walked in blocks of 64 (one
// 128-byte swizzle atom per row), double-buffered in shared memory; every thread stages 16-byte
// chunks with the 128B swizzle, one elected thread issues four UMMAs (K = 16 each) per block and
// commits them to the buffer's mbarrier; the epilogue reads the accumulator with tcgen05.ld (warp
// w owns TMEM lanes 32w..32w+31 = rows of the tile).  grid.y splits K (weight gradients, K = batch)
// with atomically accumulated FP32 output.
#include <cuda_bf16.h>

#include "mlp.cuh"
#include "umma.cuh"

namespace gbfwn {

cudaError_t prepareGemm();

namespace {

constexpr int kBM = 128, kBK = 64;

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float siluGrad(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// copy a [rows x 64] bf16 block (row stride ld elements) into a 128B-swizzled K-major tile
__device__ __forceinline__ void stageTile(uint8_t* tile, const __nv_bfloat16* src, int64_t ld, int rows) {
    for (int idx = threadIdx.x; idx < rows * 8; idx += blockDim.x) {
        const int r = idx >> 3, c = idx & 7;
        const uint4 v = *reinterpret_cast<const uint4*>(src + int64_t(r) * ld + c * 8);
        *reinterpret_cast<uint4*>(tile + r * 128 + ((c ^ (r & 7)) << 4)) = v;
    }
}

template <int N>
__global__ void __launch_bounds__(128) gemmKernel(const __nv_bfloat16* __restrict__ A, int64_t lda,
                                                  const __nv_bfloat16* __restrict__ B, int64_t ldb, int K, GemmEpilogue ep) {
    constexpr int kTmemCols = N <= 128 ? 128 : 256;
    constexpr int kTileA = kBM * 128, kTileB = N * 128;
    extern __shared__ __align__(1024) uint8_t smemRaw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
    uint8_t* tileA[2] = {smem, smem + kTileA};
    uint8_t* tileB[2] = {smem + 2 * kTileA, smem + 2 * kTileA + kTileB};
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmemBase;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t m0 = int64_t(blockIdx.x) * kBM;
    const int splits = gridDim.y;
    const int kPer = ((K / kBK + splits - 1) / splits) * kBK;
    const int kBegin = blockIdx.y * kPer, kEnd = min(K, kBegin + kPer);
    if (warp == 0) umma::tmemAlloc(&tmemBase, kTmemCols);
    if (threadIdx.x == 0) {
        umma::mbarInit(&bar[0], 1);
        umma::mbarInit(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    umma::fenceBeforeSync();
    __syncthreads();
    umma::fenceAfterSync();
    const uint32_t tmem = tmemBase;
    constexpr uint32_t idesc = umma::idescBf16(kBM, N);
    bool ok = true;
    int nb = 0;
    for (int k0 = kBegin; k0 < kEnd; k0 += kBK, ++nb) {
        const int buf = nb & 1;
        if (nb >= 2 && !umma::mbarWait(&bar[buf], ((nb - 2) >> 1) & 1)) ok = false;
        stageTile(tileA[buf], A + m0 * lda + k0, lda, kBM);
        stageTile(tileB[buf], B + k0, ldb, N);
        umma::fenceProxyAsync();
        __syncthreads();
        if (threadIdx.x == 0) {
            umma::fenceAfterSync();
            const uint32_t sa = umma::smemAddr(tileA[buf]), sb = umma::smemAddr(tileB[buf]);
            for (int kk = 0; kk < kBK / 16; ++kk)
                umma::mmaBf16(tmem, umma::descK128(sa + 32 * kk), umma::descK128(sb + 32 * kk), idesc,
                              (nb > 0 || kk > 0) ? 1u : 0u);
            umma::commit(&bar[buf]);
        }
    }
    if (nb > 0 && !umma::mbarWait(&bar[(nb - 1) & 1], ((nb - 1) >> 1) & 1)) ok = false;
    if (nb >= 2 && !umma::mbarWait(&bar[nb & 1], ((nb - 2) >> 1) & 1)) ok = false;
    umma::fenceAfterSync();
    if (!ok && ep.status && threadIdx.x == 0) atomicOr(ep.status, 2u);
    const int64_t row = m0 + 32 * warp + lane;
    if (ok && nb > 0) {
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            umma::tmemLoad16(tmem + (uint32_t(32 * warp) << 16) + uint32_t(c0), v);
            if (ep.mode == GemmEpilogue::kStoreF32) {
                float* d = ep.D + row * ep.ldd + c0;
                if (splits > 1)
                    for (int j = 0; j < 16; ++j) atomicAdd(d + j, v[j]);
                else
                    for (int j = 0; j < 16; ++j) d[j] = v[j];
            } else if (ep.mode == GemmEpilogue::kForward) {
                for (int j = 0; j < 16; ++j) {
                    const int col = c0 + j;
                    const float z = v[j] + ep.bias[col];
                    if (ep.Z) ep.Z[row * ep.ldz + col] = z;
                    const __nv_bfloat16 h = __float2bfloat16(ep.noAct ? z : silu(z));
                    if (ep.H) ep.H[row * ep.ldh + col] = h;
                    if (ep.HT) ep.HT[int64_t(col) * ep.ldht + row] = h;
                }
            } else {  // kBackward: gradient through SiLU
                for (int j = 0; j < 16; ++j) {
                    const int col = c0 + j;
                    const float g = v[j] * siluGrad(ep.Z[row * ep.ldz + col]);
                    const __nv_bfloat16 gb = __float2bfloat16(g);
                    ep.H[row * ep.ldh + col] = gb;
                    if (ep.HT) ep.HT[int64_t(col) * ep.ldht + row] = gb;
                    if (ep.dbias) {
                        float s = g;
                        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                        if (lane == 0) atomicAdd(ep.dbias + col, s);
                    }
                }
            }
        }
    }
    umma::fenceBeforeSync();
    __syncthreads();
    if (warp == 0) umma::tmemFree(tmem, kTmemCols);
}

// The timeout path of the tensor-core kernels, on purpose: a warp allocates TMEM, waits on an
// mbarrier that nothing ever arrives on with a bounded number of polls, records the timeout in the
// status word and still frees its TMEM -- what gemmKernel and inferKernel do when a wait gives up.
__global__ void __launch_bounds__(32) waitTimeoutKernel(uint32_t maxPolls, unsigned* status) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmemBase;
    umma::tmemAlloc(&tmemBase, 32);
    if (threadIdx.x == 0) {
        umma::mbarInit(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    umma::fenceBeforeSync();
    __syncthreads();
    umma::fenceAfterSync();
    const bool ok = umma::mbarWait(&bar, 0, maxPolls);  // phase 0 never completes
    if (!ok && threadIdx.x == 0) atomicOr(status, 2u);
    umma::fenceBeforeSync();
    __syncthreads();
    umma::tmemFree(tmemBase, 32);
}

template <int N> constexpr size_t gemmSmem() { return 2 * (kBM * 128 + N * 128) + 1024; }

// the dynamic shared-memory opt-in is set once per device, outside any stream capture
bool g_gemmReady[64] = {};

template <int N>
cudaError_t launchGemmN(const __nv_bfloat16* A, int64_t lda, const __nv_bfloat16* B, int64_t ldb, int M, int K, int splitK,
                        const GemmEpilogue& ep, cudaStream_t s) {
    constexpr size_t smem = gemmSmem<N>();
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !g_gemmReady[dev]) {
        cudaError_t e = prepareGemm();
        if (e) return e;
    }
    dim3 grid(unsigned(M / kBM), unsigned(splitK));
    gemmKernel<N><<<grid, 128, smem, s>>>(A, lda, B, ldb, K, ep);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launchWaitTimeout(uint32_t maxPolls, unsigned* status, cudaStream_t s) {
    waitTimeoutKernel<<<1, 32, 0, s>>>(maxPolls, status);
    return cudaGetLastError();
}

cudaError_t prepareGemm() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if ((e = cudaFuncSetAttribute(gemmKernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(gemmSmem<128>())))) return e;
    if ((e = cudaFuncSetAttribute(gemmKernel<192>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(gemmSmem<192>())))) return e;
    if (dev >= 0 && dev < 64) g_gemmReady[dev] = true;
    return cudaSuccess;
}

cudaError_t launchGemmBf16(const __nv_bfloat16* A, int64_t lda, const __nv_bfloat16* B, int64_t ldb, int M, int N, int K,
                           int splitK, const GemmEpilogue& ep, cudaStream_t s) {
    if (M <= 0 || M % kBM || K <= 0 || K % kBK || splitK < 1 || (lda % 8) || (ldb % 8)) return cudaErrorInvalidValue;
    if (splitK > 1 && ep.mode != GemmEpilogue::kStoreF32) return cudaErrorInvalidValue;
    if (N == 128) return launchGemmN<128>(A, lda, B, ldb, M, K, splitK, ep, s);
    if (N == 192) return launchGemmN<192>(A, lda, B, ldb, M, K, splitK, ep, s);
    return cudaErrorInvalidValue;
}

}  // namespace gbfwn
