// tcgen05 (5th-generation tensor core) building blocks for sm_103a, written as inline PTX:
// TMEM allocation, shared-memory matrix descriptors (K-major, 128-byte swizzle), the BF16 UMMA
// with FP32 accumulation in TMEM, commit to an mbarrier, bounded mbarrier waits, and TMEM loads.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace gbfwn {
namespace umma {

__device__ __forceinline__ uint32_t smemAddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor for a K-major operand tile stored with the 128-byte swizzle:
// rows of 64 bf16 (128 bytes), 8-row atoms of 1024 bytes stacked along M/N (stride 1024 bytes),
// 16-byte chunk c of row r stored at chunk position c ^ (r % 8).  The tile base must be
// 1024-byte aligned; stepping K by 16 elements inside the atom advances the start address by 32
// bytes.  Fields: start address >> 4 [0,14), leading byte offset >> 4 [16,30) (unused for this
// layout), stride byte offset >> 4 [32,46), descriptor version 1 [46,48), layout type
// SWIZZLE_128B = 2 [61,64).
__device__ __forceinline__ uint64_t descK128(uint32_t saddr) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3ffffu) >> 4);
    d |= uint64_t(1) << 16;
    d |= uint64_t(1024 >> 4) << 32;
    d |= uint64_t(1) << 46;
    d |= uint64_t(2) << 61;
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: D = FP32 [4,6) = 1, A = BF16 [7,10) = 1,
// B = BF16 [10,13) = 1, both K-major (bits 15, 16 = 0), N >> 3 at [17,23), M >> 4 at [24,29).
__host__ __device__ constexpr uint32_t idescBf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void mmaBf16(uint32_t tmemD, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmemD),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Arrive once on the mbarrier when all previously issued MMAs of this thread have completed.
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smemAddr(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbarInit(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smemAddr(mbar)), "r"(count) : "memory");
}

// Waits for phase `parity` of the mbarrier to complete; gives up after `maxIter` polls and
// returns false (the caller records the timeout instead of hanging).
__device__ __forceinline__ bool mbarWait(uint64_t* mbar, uint32_t parity, uint32_t maxIter = 1u << 22) {
    const uint32_t a = smemAddr(mbar);
    for (uint32_t it = 0; it < maxIter; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// TMEM allocation by one full warp; the allocated column base is written to *dst (shared memory).
__device__ __forceinline__ void tmemAlloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}

__device__ __forceinline__ void tmemFree(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// make generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape: thread i of the warp
// reads lane (warp's quadrant base + i)).
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// The same load without the wait: issue several, then tmemWaitLoads16 on each destination array
// (the wait names the registers, so no use of them can be scheduled before it).
__device__ __forceinline__ void tmemLoad16Async(uint32_t taddr, uint32_t r[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmemWaitLoads16(uint32_t r[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;\n"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]),
                   "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])
                 :
                 : "memory");
}

// 32 consecutive FP32 TMEM columns of this thread's lane: two loads, one tied wait each.
__device__ __forceinline__ void tmemLoad32(uint32_t taddr, float v[32]) {
    uint32_t r[32];
    tmemLoad16Async(taddr, r);
    tmemLoad16Async(taddr + 16, r + 16);
    tmemWaitLoads16(r);
    tmemWaitLoads16(r + 16);
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// TMA bulk copy global -> shared completing on mbarrier `bar`, issued by one thread: arms the
// barrier with the byte count, then copies in pieces of at most 16 KB (addresses 16-byte aligned,
// bytes a multiple of 16).
__device__ __forceinline__ void bulkLoad(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    constexpr uint32_t kPiece = 16384;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smemAddr(bar)), "r"(bytes) : "memory");
    for (uint32_t o = 0; o < bytes; o += kPiece)
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                         smemAddr(static_cast<uint8_t*>(dst) + o)),
                     "l"(static_cast<const uint8_t*>(src) + o), "r"(bytes - o < kPiece ? bytes - o : kPiece), "r"(smemAddr(bar))
                     : "memory");
}

// TMA bulk copy shared -> global (one thread), committed as a bulk group.
__device__ __forceinline__ void bulkStore(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst), "r"(smemAddr(src)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
}

}  // namespace umma
}  // namespace gbfwn
