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

// ---------------------------------------------------------------- network layout
// Fourier features -> 4 x (128, SiLU) -> 1; parameters (FP32) W1[128 x 192] b1 W2[128 x 128] b2 W3 b3 W4 b4 w5[128] b5.
constexpr int kMlpF = 192, kMlpH = 128, kMlpFreq = 32;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kMlpH * kMlpF, kOffW2 = kOffB1 + kMlpH, kOffB2 = kOffW2 + kMlpH * kMlpH,
              kOffW3 = kOffB2 + kMlpH, kOffB3 = kOffW3 + kMlpH * kMlpH, kOffW4 = kOffB3 + kMlpH,
              kOffB4 = kOffW4 + kMlpH * kMlpH, kOffW5 = kOffB4 + kMlpH, kOffB5 = kOffW5 + kMlpH;

// The bf16 hidden-layer weights as shared-memory images: 9 blocks of 16 KB, each a 128-row x 64-column
// K-major tile with the 128-byte swizzle (row r at r * 128 bytes, 16-byte chunk c at position
// c ^ (r % 8)): W1 blocks 0..2 (input columns 0..191), W2 blocks 3..4, W3 5..6, W4 7..8.  A block is
// copied into shared memory as it is (one bulk copy) and read there by the tensor cores.
constexpr int kImgBlockBytes = 128 * 128;
constexpr int kImgBlocks = 9;

struct NetMeta;

// One fused training step (mlp_train.cu): forward, loss and backward of nPad rows (a multiple of 128;
// rows >= n are padding and contribute nothing), 128 rows per CTA; parameter gradients are added
// into `grads` and the mean squared error into `loss` (both zeroed by the caller).
struct TrainStepArgs {
    const float* pts;
    const float* targets;
    const int32_t* idx;     // rows are idx[(*offPtr + i) % idxMod] when idx is not null
    const int32_t* offPtr;
    int64_t idxMod;
    int n, nPad;
    float clampD;
    const float* params;
    const __nv_bfloat16* img;   // kImgBlocks weight images
    __nv_bfloat16* spill;       // 32 KB per CTA: the first hidden layer's activations between uses
    float* grads;
    float* loss;
    unsigned* status;           // bit 1: a bounded wait gave up
};
cudaError_t prepareTrainStep();
cudaError_t launchTrainStep(const TrainStepArgs& a, const NetMeta& meta, cudaStream_t s);

}  // namespace gbfwn
