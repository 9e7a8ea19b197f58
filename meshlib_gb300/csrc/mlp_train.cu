// One training step of the surrogate network fused into one kernel on the 5th-generation tensor
// cores: features, the four hidden layers, the output layer and loss, and the whole backward pass
// for 128 rows per CTA, without leaving the SM except for the weights (bulk-copied from L2 as
// pre-swizzled shared-memory images), one 32 KB activation spill and the gradient reduction.
//
// Rounding points are those of the network's definition (oracle/mlp_oracle.py restates them):
// features, weights, hidden activations and the activation gradients that feed the tensor cores in
// bf16; pre-activations, accumulators, bias / output-layer gradients and the weight gradients in FP32.
//
// Shared-memory tiles are 128-row K-major tiles with the 128-byte swizzle (64-column blocks of 16 KB).
// The same tile is read as a K-major operand by one GEMM and as the transposed (MN-major) operand of
// another, so no transposed copies exist:
//   forward   Z_l  = H_{l-1} W_l^T          A = H_{l-1} (K-major)   B = W_l (K-major)
//   backward  dH_{l-1} = dZ_l W_l           A = dZ_l (K-major)      B = W_l (MN-major)
//             dW_l = dZ_l^T H_{l-1}         A = dZ_l (MN-major)     B = H_{l-1} (MN-major), K = rows
// TMEM (512 columns): Z1..Z4 at columns 0 / 128 / 256 / 384 after the forward pass; each backward
// epilogue frees the block it has consumed for the next accumulators.
#include <cuda_bf16.h>

#include <cstdint>

#include "common.cuh"
#include "mlp.cuh"
#include "surrogate.cuh"
#include "mlp_tiles.cuh"
#include "umma.cuh"

namespace gbfwn {

namespace {

using mlp::loadParams16;
using mlp::packBf16x2;
using mlp::storeRow16;
using umma::bulkLoad;
using umma::bulkStore;
using umma::tmemLoad32;
__device__ __forceinline__ float siluf(float z) { return mlp::silu(z); }
__device__ __forceinline__ float siluGradf(float z) { return mlp::siluGrad(z); }

constexpr int kT = 512;                 // 16 warps: TMEM lane quarter (warp % 4) x column quarter (warp / 4)
constexpr int kParts = kT / 128;        // threads per row in the epilogues (and in the feature pass)
constexpr uint32_t kBlk = kImgBlockBytes;  // 16 KB: 128 rows x 64 bf16 columns
// slots of the dynamic shared memory (offsets from its 1024-byte aligned base)
constexpr uint32_t kX0 = 0, kX1 = 3 * kBlk, kY0 = 6 * kBlk, kY1 = 8 * kBlk, kY2 = 10 * kBlk, kY3 = 12 * kBlk;
constexpr uint32_t kTrainSmem = 14 * kBlk + 1024;
constexpr uint32_t FULLMASK = 0xffffffffu;
constexpr uint32_t kMaxPolls = 1u << 22;

// Shared-memory descriptor of a transposed (MN-major) operand read from a 128-row K-major tile: the
// tile's 64-column blocks are the 64-element MN atoms (leading byte offset = block size), its 8-row
// groups are the K groups (stride byte offset 1024); 128-byte swizzle, descriptor version 1.
__device__ __forceinline__ uint64_t descMN128(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3ffffu) >> 4);
    d |= uint64_t(kBlk >> 4) << 16;
    d |= uint64_t(1024 >> 4) << 32;
    d |= uint64_t(1) << 46;
    d |= uint64_t(2) << 61;
    return d;
}

// one thread: D[tmem] = A * B^T over K (multiple of 16), M = 128, N columns; operands in shared memory
__device__ __forceinline__ void mmaTile(uint32_t tmem, uint32_t a, bool aMN, uint32_t b, bool bMN, int N, int K) {
    const uint32_t idesc = umma::idescBf16(128, N) | (aMN ? 1u << 15 : 0u) | (bMN ? 1u << 16 : 0u);
    for (int s = 0; s < K / 16; ++s) {
        const uint64_t da = aMN ? descMN128(a + 2048u * s) : umma::descK128(a + uint32_t(s / 4) * kBlk + 32u * (s % 4));
        const uint64_t db = bMN ? descMN128(b + 2048u * s) : umma::descK128(b + uint32_t(s / 4) * uint32_t(N) * 128u + 32u * (s % 4));
        umma::mmaBf16(tmem, da, db, idesc, s > 0 ? 1u : 0u);
    }
}

__device__ __forceinline__ void redAdd4(float* p, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};\n" ::"l"(p), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

// Sum over the warp's 32 lanes of 16 per-lane values: afterwards lane L holds the sum of column
// (L >> 1) & 15 (each column twice, in lanes 2c and 2c + 1).  16 shuffles instead of 80.
__device__ __forceinline__ float warpColumnSum16(float v[16], int lane) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const bool up = lane & 16;
        const float send = up ? v[j] : v[j + 8], keep = up ? v[j + 8] : v[j];
        v[j] = keep + __shfl_xor_sync(FULLMASK, send, 16);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const bool up = lane & 8;
        const float send = up ? v[j] : v[j + 4], keep = up ? v[j + 4] : v[j];
        v[j] = keep + __shfl_xor_sync(FULLMASK, send, 8);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const bool up = lane & 4;
        const float send = up ? v[j] : v[j + 2], keep = up ? v[j + 2] : v[j];
        v[j] = keep + __shfl_xor_sync(FULLMASK, send, 4);
    }
    {
        const bool up = lane & 2;
        const float send = up ? v[0] : v[1], keep = up ? v[1] : v[0];
        v[0] = keep + __shfl_xor_sync(FULLMASK, send, 2);
    }
    return v[0] + __shfl_xor_sync(FULLMASK, v[0], 1);
}

struct Sync {
    uint64_t* mma;
    uint32_t phase = 0;
    int* failed;
    // every thread: wait for the MMAs committed last, then order the tensor core's TMEM writes before
    // the epilogue's loads
    __device__ __forceinline__ void waitMma() {
        if (!umma::mbarWait(mma, phase, kMaxPolls)) atomicOr(failed, 1);
        phase ^= 1u;
        umma::fenceAfterSync();
    }
};

// all threads: make this phase's shared-memory writes visible to the tensor core and end the phase
__device__ __forceinline__ void endPhase() {
    umma::fenceProxyAsync();
    umma::fenceBeforeSync();
    __syncthreads();
    umma::fenceAfterSync();
}

// Features of this CTA's rows into the 48 KB K-major tile F (axis a = block a; column 2k / 2k + 1 =
// sin / cos of frequency k): thread (row, part) writes frequencies 8 part .. 8 part + 7.
__device__ void featuresTile(uint8_t* F, const TrainStepArgs& a, const NetMeta& meta, int rowBase) {
    const int t = threadIdx.x, row = t & 127, fh = t >> 7;
    constexpr int kChunks = 8 / kParts;  // 16-byte chunks (4 frequencies each, 8 per axis) per thread and axis
    static_assert(kChunks * kParts == 8, "every chunk of every axis written once");
    const int i = rowBase + row;
    float u[3] = {0.f, 0.f, 0.f};
    if (i < a.n) {
        int64_t j = i;
        if (a.idx) j = a.idx[(int64_t(a.offPtr ? *a.offPtr : 0) + i) % a.idxMod];
        for (int ax = 0; ax < 3; ++ax) u[ax] = (a.pts[3 * j + ax] - meta.center[ax]) * meta.scale;
    }
    const bool live = i < a.n;
    for (int ax = 0; ax < 3; ++ax)
        for (int c = kChunks * fh; c < kChunks * fh + kChunks; ++c) {
            uint32_t w[4];
            for (int q = 0; q < 4; ++q) {
                float sv = 0.f, cv = 0.f;
                if (live) sincosf(meta.freq[4 * c + q] * u[ax], &sv, &cv);
                w[q] = packBf16x2(sv, cv);
            }
            *reinterpret_cast<uint4*>(F + ax * kBlk + row * 128 + ((c ^ (row & 7)) << 4)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
}

__global__ void __launch_bounds__(kT, 1) trainStepKernel(TrainStepArgs a, NetMeta meta) {
    extern __shared__ __align__(1024) uint8_t smemRaw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
    uint8_t *X0 = sm + kX0, *X1 = sm + kX1, *Y0 = sm + kY0, *Y1 = sm + kY1, *Y2 = sm + kY2, *Y3 = sm + kY3;
    __shared__ __align__(8) uint64_t barMma, barX0, barY0, barY2;
    __shared__ uint32_t tmemBase;
    __shared__ int failed;
    // column sums of the epilogues (colA, colB); the output layer's per-row partial dot products
    // use the same 1 KB before its column sums start (the tiles take all but ~2 KB of the 227 KB)
    __shared__ float colBuf[256];  // kT >= 256
    __shared__ float blockSum[2];
    float* colA = colBuf;
    float* colB = colBuf + 128;
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int q = warp & 3, hf = warp >> 2;  // hf: this thread's column part (of kParts)
    const int row = 32 * q + lane;  // this thread's row in every epilogue
    const int rowBase = blockIdx.x * 128;
    const int gRow = rowBase + row;
    const __nv_bfloat16* img = a.img;
    uint8_t* spill = reinterpret_cast<uint8_t*>(a.spill) + size_t(blockIdx.x) * 2 * kBlk;

    if (warp == 0) umma::tmemAlloc(&tmemBase, 512);
    if (t == 0) {
        umma::mbarInit(&barMma, 1);
        umma::mbarInit(&barX0, 1);
        umma::mbarInit(&barY0, 1);
        umma::mbarInit(&barY2, 1);
        failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (t < 256) colBuf[t] = 0.f;
    if (t < 2) blockSum[t] = 0.f;
    umma::fenceBeforeSync();
    __syncthreads();
    umma::fenceAfterSync();
    const uint32_t tmem = tmemBase;
    const uint32_t tq = tmem + (uint32_t(32 * q) << 16);  // this warp's TMEM lane quarter
    Sync sy{&barMma, 0u, &failed};
    uint32_t phX0 = 0, phY0 = 0;  // next completion parity of the load barriers

    auto waitLoad = [&](uint64_t* bar, uint32_t& ph) {  // thread 0 only
        if (!umma::mbarWait(bar, ph, kMaxPolls)) atomicOr(&failed, 1);
        ph ^= 1u;
    };
    // column sums of the rows of a 16-column group into colX[c0 .. c0 + 15]
    auto colAdd = [&](float* colX, int c0, float v[16]) {
        const float s = warpColumnSum16(v, lane);
        if ((lane & 1) == 0) atomicAdd(&colX[c0 + ((lane >> 1) & 15)], s);
    };
    // forward epilogue of hidden layer l (1..3): H_l = bf16(silu(Z_l + b_l)) into tile `out`
    auto forwardEpilogue = [&](int l, uint8_t* out) {
        const float* bias = a.params + (l == 1 ? kOffB1 : l == 2 ? kOffB2 : kOffB3);
        const int cb = 32 * hf;
        float v[32];
        tmemLoad32(tq + uint32_t(128 * (l - 1) + cb), v);
        for (int h = 0; h < 2; ++h) {
            float b[16];
            loadParams16(bias + cb + 16 * h, b);
            uint32_t w[8];
            for (int j = 0; j < 16; j += 2)
                w[j / 2] = packBf16x2(siluf(v[16 * h + j] + b[j]), siluf(v[16 * h + j + 1] + b[j + 1]));
            storeRow16(out, row, cb + 16 * h, w);
        }
    };
    // backward epilogue: dZ_{l} = bf16(dH * silu'(Z_l + b_l)) into tile `out` from dH at TMEM column
    // 384 and Z_l at 128 (l - 1); bias gradient sums into colA
    auto backwardEpilogue = [&](int l, uint8_t* out) {
        const float* bias = a.params + (l == 1 ? kOffB1 : l == 2 ? kOffB2 : kOffB3);
        const int cb = 32 * hf;
        for (int h = 0; h < 2; ++h) {
            const int c0 = cb + 16 * h;
            uint32_t rg[16], rz[16];
            umma::tmemLoad16Async(tq + uint32_t(384 + c0), rg);
            umma::tmemLoad16Async(tq + uint32_t(128 * (l - 1) + c0), rz);
            umma::tmemWaitLoads16(rg);
            umma::tmemWaitLoads16(rz);
            float b[16], g[16];
            loadParams16(bias + c0, b);
            uint32_t w[8];
            for (int j = 0; j < 16; ++j) g[j] = __uint_as_float(rg[j]) * siluGradf(__uint_as_float(rz[j]) + b[j]);
            for (int j = 0; j < 16; j += 2) w[j / 2] = packBf16x2(g[j], g[j + 1]);
            storeRow16(out, row, c0, w);
            colAdd(colA, c0, g);
        }
    };
    // gradient of W_l from TMEM column `col` (N columns of input per row = output unit `row`)
    auto weightGradEpilogue = [&](uint32_t col, int N, int off) {
        const int part = N / kParts;  // 32 (N = 128) or 48 (N = 192) columns per thread
        for (int c0 = part * hf; c0 < part * hf + part; c0 += 16) {
            float v[16];
            umma::tmemLoad16(tq + col + uint32_t(c0), v);
            float* g = a.grads + off + int64_t(row) * N + c0;
            for (int j = 0; j < 16; j += 4) redAdd4(g + j, v[j], v[j + 1], v[j + 2], v[j + 3]);
        }
    };
    // colA (and colB) -> the gradient entries; then cleared for the next use
    auto flushCols = [&](int offA, int offB) {
        __syncthreads();
        if (t < 128) {
            atomicAdd(&a.grads[offA + t], colA[t]);
            colA[t] = 0.f;
            if (offB >= 0) {
                atomicAdd(&a.grads[offB + t], colB[t]);
                colB[t] = 0.f;
            }
        }
    };

    // ---------------------------------------------------------------- forward
    if (t == 0) {
        bulkLoad(X0, img, 3 * kBlk, &barX0);            // W1
        bulkLoad(Y0, img + 3 * kBlk / 2, 2 * kBlk, &barY0);  // W2
    }
    featuresTile(X1, a, meta, rowBase);
    endPhase();
    if (t == 0) {
        waitLoad(&barX0, phX0);
        umma::fenceAfterSync();
        mmaTile(tmem + 0, umma::smemAddr(X1), false, umma::smemAddr(X0), false, 128, kMlpF);
        umma::commit(&barMma);
    }
    sy.waitMma();
    forwardEpilogue(1, Y1);  // H1
    endPhase();
    if (t == 0) {
        bulkLoad(X0, img + 5 * kBlk / 2, 2 * kBlk, &barX0);  // W3 (W1 is done)
        waitLoad(&barY0, phY0);
        umma::fenceAfterSync();
        mmaTile(tmem + 128, umma::smemAddr(Y1), false, umma::smemAddr(Y0), false, 128, kMlpH);
        umma::commit(&barMma);
    }
    sy.waitMma();
    forwardEpilogue(2, X1);  // H2 (F is done)
    endPhase();
    if (t == 0) {
        bulkStore(spill, Y1, 2 * kBlk);                       // H1 until dW2
        bulkLoad(Y0, img + 7 * kBlk / 2, 2 * kBlk, &barY0);   // W4 (W2 is done)
        waitLoad(&barX0, phX0);
        umma::fenceAfterSync();
        mmaTile(tmem + 256, umma::smemAddr(X1), false, umma::smemAddr(X0), false, 128, kMlpH);
        umma::commit(&barMma);
    }
    sy.waitMma();
    forwardEpilogue(3, Y2);  // H3
    endPhase();
    if (t == 0) {
        waitLoad(&barY0, phY0);
        umma::fenceAfterSync();
        mmaTile(tmem + 384, umma::smemAddr(Y2), false, umma::smemAddr(Y0), false, 128, kMlpH);
        umma::commit(&barMma);
        asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");  // Y1 may be overwritten after this phase
    }
    sy.waitMma();
    // ---------------------------------------------------------------- output layer and loss
    {
        const float* b4 = a.params + kOffB4;
        const float* w5 = a.params + kOffW5;
        const int cb = 32 * hf;
        float z4[32], b4v[32], w5v[32];
        tmemLoad32(tq + uint32_t(384 + cb), z4);
        loadParams16(b4 + cb, b4v);
        loadParams16(b4 + cb + 16, b4v + 16);
        loadParams16(w5 + cb, w5v);
        loadParams16(w5 + cb + 16, w5v + 16);
        float acc = 0.f;
        for (int j = 0; j < 32; ++j) {
            z4[j] += b4v[j];
            acc += __bfloat162float(__float2bfloat16(siluf(z4[j]))) * w5v[j];
        }
        // per-row partial dot products of the kParts column parts, in the spilled tile's slot (its
        // bulk store has read it: thread 0 waited for that before this phase, hence the barrier)
        float* rowPart = reinterpret_cast<float*>(Y1);
        __syncthreads();
        rowPart[128 * hf + row] = acc;
        __syncthreads();
        float ysum = a.params[kOffB5];
        for (int p2 = 0; p2 < kParts; ++p2) ysum += rowPart[128 * p2 + row];
        const float y = ysum;
        float g = 0.f, l2 = 0.f;
        if (gRow < a.n) {
            int64_t j = gRow;
            if (a.idx) j = a.idx[(int64_t(a.offPtr ? *a.offPtr : 0) + gRow) % a.idxMod];
            const float tg = fminf(fmaxf(a.targets[j], -a.clampD), a.clampD);
            const float r = y - tg;
            const float invN = 1.f / float(a.n);
            g = 2.f * r * invN;
            l2 = r * r * invN;
        }
        if (hf == 0) {  // warp-uniform: one of the kParts threads of each row counts it
            float gs = g;
            for (int o = 16; o; o >>= 1) {
                l2 += __shfl_xor_sync(FULLMASK, l2, o);
                gs += __shfl_xor_sync(FULLMASK, gs, o);
            }
            if (lane == 0) {
                atomicAdd(&blockSum[0], l2);
                atomicAdd(&blockSum[1], gs);
            }
        }
        for (int h = 0; h < 2; ++h) {
            const int c0 = cb + 16 * h;
            float v[16], gw[16];
            uint32_t w[8];
            for (int jj = 0; jj < 16; ++jj) {
                const float z = z4[16 * h + jj];
                gw[jj] = g * __bfloat162float(__float2bfloat16(siluf(z)));  // w5 gradient term
                v[jj] = g * w5v[16 * h + jj] * siluGradf(z);                // dZ4 (FP32)
            }
            for (int jj = 0; jj < 16; jj += 2) w[jj / 2] = packBf16x2(v[jj], v[jj + 1]);
            storeRow16(Y3, row, c0, w);
            colAdd(colA, c0, v);   // b4
            colAdd(colB, c0, gw);  // w5
        }
        flushCols(kOffB4, kOffW5);
        if (t == 0) {
            atomicAdd(a.loss, blockSum[0]);
            atomicAdd(&a.grads[kOffB5], blockSum[1]);
        }
    }
    endPhase();
    // ---------------------------------------------------------------- backward
    if (t == 0) {  // dH3 = dZ4 W4
        mmaTile(tmem + 384, umma::smemAddr(Y3), false, umma::smemAddr(Y0), true, 128, kMlpH);
        umma::commit(&barMma);
    }
    sy.waitMma();
    backwardEpilogue(3, Y1);  // dZ3
    flushCols(kOffB3, -1);
    endPhase();
    if (t == 0) {  // dW4 = dZ4^T H3; dH2 = dZ3 W3
        mmaTile(tmem + 256, umma::smemAddr(Y3), true, umma::smemAddr(Y2), true, 128, 128);
        mmaTile(tmem + 384, umma::smemAddr(Y1), false, umma::smemAddr(X0), true, 128, kMlpH);
        umma::commit(&barMma);
    }
    sy.waitMma();
    if (t == 0) {  // W4, H3, dZ4, W3 are done: W2 and the spilled H1 come back
        bulkLoad(Y0, img + 3 * kBlk / 2, 2 * kBlk, &barY0);
        asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
        bulkLoad(Y2, spill, 2 * kBlk, &barY2);
    }
    weightGradEpilogue(256, 128, kOffW4);
    backwardEpilogue(2, Y3);  // dZ2
    flushCols(kOffB2, -1);
    endPhase();
    uint32_t phY2 = 0;
    if (t == 0) {  // dW3 = dZ3^T H2; dH1 = dZ2 W2
        mmaTile(tmem + 256, umma::smemAddr(Y1), true, umma::smemAddr(X1), true, 128, 128);
        waitLoad(&barY0, phY0);
        umma::fenceAfterSync();
        mmaTile(tmem + 384, umma::smemAddr(Y3), false, umma::smemAddr(Y0), true, 128, kMlpH);
        umma::commit(&barMma);
    }
    sy.waitMma();
    featuresTile(X1, a, meta, rowBase);  // F again (H2 is done), for dW1
    weightGradEpilogue(256, 128, kOffW3);
    backwardEpilogue(1, Y1);  // dZ1 (dZ3 is done)
    flushCols(kOffB1, -1);
    endPhase();
    if (t == 0) {  // dW2 = dZ2^T H1; dW1 = dZ1^T F
        waitLoad(&barY2, phY2);
        umma::fenceAfterSync();
        mmaTile(tmem + 256, umma::smemAddr(Y3), true, umma::smemAddr(Y2), true, 128, 128);
        mmaTile(tmem + 0, umma::smemAddr(Y1), true, umma::smemAddr(X1), true, kMlpF, 128);
        umma::commit(&barMma);
    }
    sy.waitMma();
    weightGradEpilogue(256, 128, kOffW2);
    weightGradEpilogue(0, kMlpF, kOffW1);
    umma::fenceBeforeSync();
    __syncthreads();
    if (t == 0 && failed && a.status) atomicOr(a.status, 2u);
    if (warp == 0) umma::tmemFree(tmem, 512);
}

}  // namespace

cudaError_t prepareTrainStep() {
    return cudaFuncSetAttribute(trainStepKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kTrainSmem));
}

cudaError_t launchTrainStep(const TrainStepArgs& a, const NetMeta& meta, cudaStream_t s) {
    if (a.nPad <= 0 || a.nPad % 128 || a.n > a.nPad) return cudaErrorInvalidValue;
    trainStepKernel<<<unsigned(a.nPad / 128), kT, kTrainSmem, s>>>(a, meta);
    return cudaGetLastError();
}

}  // namespace gbfwn
