// Blackwell (sm_103a) tensor-core helpers: tcgen05.mma with FP32 accumulators
// in tensor memory (TMEM), shared-memory matrix descriptors of the
// no-swizzle canonical K-major layout, mbarrier completion with bounded
// waits, bulk copies (cp.async.bulk) into shared memory, and the TF32
// splitting that lets three TF32 products carry FP32 operands
// (x = hi + lo, hi = x rounded to TF32, lo = x - hi rounded to TF32;
// x y ~ hi_x hi_y + hi_x lo_y + lo_x hi_y, relative error ~2^-21).
//
// Operand layout in shared memory (K-major, no swizzle): an R x K FP32
// operand is stored as 8-row x 16-byte core matrices (8 rows of 4 elements,
// 128 contiguous bytes); core matrix (i, kk) -- rows 8i..8i+7, elements
// 4kk..4kk+3 of K -- sits at byte ((i * KC) + kk) * 128 with KC = K / 4.
// Its descriptor has the leading-dimension byte offset (between core
// matrices along K) 128 and the stride-dimension offset (between 8-row
// groups) KC * 128; one MMA of K = 8 (32 bytes) reads two core-matrix
// columns, the next MMA starts 256 bytes further.
#pragma once

#include <cstdint>

namespace lp {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) of a K-major operand with KC core columns
__host__ __device__ __forceinline__ int core_off(int row, int k, int KC) {
    return ((row >> 3) * KC + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4;
}

// shared-memory matrix descriptor: start, leading / stride byte offsets,
// descriptor version 1, base offset 0, SWIZZLE_NONE
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, M x N (M in {64, 128}, N a multiple of 16 up to 256 for M = 128)
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D (TMEM) (+)= A (smem) * B (smem)^T, issued by one thread
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)acc));
}

// arrive on the mbarrier once every MMA issued so far by this thread completes
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        smem_u32(mbar)));
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count));
}

// expect `bytes` of bulk-copy data on the mbarrier and arrive once
__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes));
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// one arrival of this thread (release: its earlier shared-memory accesses
// are ordered before the phase completes)
__device__ __forceinline__ void mbar_arrive(uint64_t *mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// named barrier `id` (1..15) over `count` threads (a multiple of 32)
__device__ __forceinline__ void named_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Wait for the completion of phase `parity`, bounded in time: the
// non-blocking test_wait is polled until the phase completes or `limit_ns`
// of the global timer have passed (false: the wait ran out).
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint64_t limit_ns = 2000000000ull) {
    const uint64_t t0 = global_ns();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (global_ns() - t0 > limit_ns) return false;
        __nanosleep(32);
    }
}

// The same wait with mbarrier.try_wait: the thread is suspended until the
// phase completes or `hint_ns` pass (then it asks again), so a waiting warp
// neither spins on the issue slots nor oversleeps the completion.
__device__ __forceinline__ bool mbar_wait_susp(uint64_t *mbar, uint32_t parity,
                                               uint64_t limit_ns = 2000000000ull, uint32_t hint_ns = 1000000u) {
    uint64_t t0 = 0;
    for (int it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity), "r"(hint_ns)
            : "memory");
        if (done) return true;
        if (it == 0) t0 = global_ns();
        else if (global_ns() - t0 > limit_ns) return false;
    }
}

// 1-D bulk copy global -> shared (16-byte aligned addresses, size a multiple
// of 16), completing on the mbarrier's transaction count
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(mbar))
                 : "memory");
}

// TMEM allocation by one full warp (the address is written to *slot)
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;"); }
// make generic-proxy shared-memory writes visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;"); }

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape: warp
// w of a warpgroup reads lanes 32 (w % 4) .. + 31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// x rounded to TF32 (round to nearest, ties away), as an FP32 bit pattern
__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

}  // namespace tc
}  // namespace lp
