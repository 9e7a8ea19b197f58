// Element-wise pieces shared by the surrogate network's fused kernels (training step and inference):
// the SiLU arithmetic, bf16 packing, vector parameter loads and writes into 128-row K-major tiles with
// the 128-byte swizzle (64-column blocks of 16 KB: row r at r * 128 bytes, 16-byte chunk c at
// position c ^ (r % 8)).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace gbfwn {
namespace mlp {

constexpr uint32_t kTileBlock = 128 * 128;  // one 128-row x 64-column bf16 block

__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.f + __expf(-z)); }
__device__ __forceinline__ float siluGrad(float z) {
    const float s = __fdividef(1.f, 1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

__device__ __forceinline__ uint32_t packBf16x2(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// 16 consecutive FP32 parameters (p 16-byte aligned) through the read-only path
__device__ __forceinline__ void loadParams16(const float* p, float v[16]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float4 x = __ldg(reinterpret_cast<const float4*>(p) + i);
        v[4 * i] = x.x;
        v[4 * i + 1] = x.y;
        v[4 * i + 2] = x.z;
        v[4 * i + 3] = x.w;
    }
}

// 16 bf16 values (8 packed words) of row r, columns c0..c0+15 (c0 % 16 == 0), into a tile
__device__ __forceinline__ void storeRow16(uint8_t* tile, int r, int c0, const uint32_t w[8]) {
    uint8_t* dst = tile + (c0 / 64) * kTileBlock + r * 128;
    const int ca = (c0 % 64) / 8;
    *reinterpret_cast<uint4*>(dst + ((ca ^ (r & 7)) << 4)) = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(dst + (((ca + 1) ^ (r & 7)) << 4)) = make_uint4(w[4], w[5], w[6], w[7]);
}

}  // namespace mlp
}  // namespace gbfwn
