// Surrogate signed-distance network (C ABI part): diagnostics of the tensor-core GEMM.
#include <cuda_bf16.h>

#include "../../include/gbfwn.h"
#include "mlp.cuh"

using namespace gbfwn;

extern "C" GBFWN_API int gbfwn_debug_gemm_bf16(const void* d_a, const void* d_b, float* d_d, int32_t m, int32_t n, int32_t k,
                                               int32_t split_k, void* stream) {
    if (!d_a || !d_b || !d_d) return GBFWN_INVALID;
    GemmEpilogue ep;
    ep.mode = GemmEpilogue::kStoreF32;
    ep.D = d_d;
    ep.ldd = n;
    const cudaError_t e = launchGemmBf16(static_cast<const __nv_bfloat16*>(d_a), k, static_cast<const __nv_bfloat16*>(d_b), k, m,
                                         n, k, split_k, ep, static_cast<cudaStream_t>(stream));
    if (e == cudaErrorInvalidValue) return GBFWN_INVALID;
    return e ? GBFWN_CUDA_ERROR : GBFWN_OK;
}
