// Surrogate network: tcgen05 GEMM interface and the network layout shared by training and
// inference.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbfwn {

struct GemmEpilogue {
    enum Mode : int { kStoreF32 = 0, kForward = 1, kBackward = 2 };
    int mode = kStoreF32;
    // kStoreF32: D[row * ldd + col] (atomically accumulated when K is split)
    float* D = nullptr;
    int64_t ldd = 0;
    // kForward: z = acc + bias[col]; Z <- z (optional); H, HT <- silu(z) (or z if noAct) in bf16
    // kBackward: g = acc * silu'(Z[row, col]); H, HT <- g in bf16; dbias[col] += sum over rows of g
    const float* bias = nullptr;
    float* Z = nullptr;
    int64_t ldz = 0;
    __nv_bfloat16* H = nullptr;
    int64_t ldh = 0;
    __nv_bfloat16* HT = nullptr;  // transposed copy: HT[col * ldht + row]
    int64_t ldht = 0;
    float* dbias = nullptr;
    int noAct = 0;
    unsigned* status = nullptr;  // bit 1: an mbarrier wait timed out
};

// D = A[M x K] * B[N x K]^T with A, B K-major bf16 (lda, ldb multiples of 8 elements, 16-byte
// aligned rows), M % 128 == 0, N in {128, 192}, K % 64 == 0.
// Sets the kernels' shared-memory opt-in on the current device (done automatically on first use;
// call it before capturing GEMMs into a CUDA graph).
cudaError_t prepareGemm();

// Runs one warp that waits on an mbarrier nothing arrives on (at most maxPolls polls), sets bit 1 of
// *status when the wait gives up, and frees its TMEM: the tensor-core kernels' timeout path.
cudaError_t launchWaitTimeout(uint32_t maxPolls, unsigned* status, cudaStream_t s);

cudaError_t launchGemmBf16(const __nv_bfloat16* A, int64_t lda, const __nv_bfloat16* B, int64_t ldb, int M, int N, int K,
                           int splitK, const GemmEpilogue& ep, cudaStream_t s);

}  // namespace gbfwn
