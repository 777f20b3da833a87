// Thin inline-PTX wrappers for the sm_100-family tensor-core path (tcgen05, TMEM, mbarrier).
//
// Operand layouts used here (PTX ISA, "tcgen05 Matrix Descriptors"):
//  * shared-memory operands are K-major, no swizzle: 8-row x 16-byte core matrices stored
//    as 128 contiguous bytes; core matrices adjacent in K are LBO bytes apart, groups of
//    8 rows SBO bytes apart.  canon_off() gives the float offset of element (row, k).
//  * TMEM: an M=128 accumulator row r is TMEM lane r, FP32 column c is TMEM column c; a
//    warp reaches the 32 lanes of its quadrant (warp id mod 4).
#pragma once

#include <cstdint>

namespace dgx {
namespace tc {

// float offset of (row, k) in a K-major no-swizzle operand with K columns (K % 4 == 0),
// LBO = 128 bytes (next 4 k), SBO = K/4 * 128 bytes (next 8 rows)
__host__ __device__ constexpr int canon_off(int row, int k, int K) {
    return (row >> 3) * (K / 4) * 32 + (k >> 2) * 32 + (row & 7) * 4 + (k & 3);
}

// shared-memory matrix descriptor (version 1, no swizzle)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFF) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::tf32: FP32 accumulator, TF32 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// D (TMEM) (+)= A (shared) * B (shared)^T
__device__ __forceinline__ void mma_ss(uint32_t d, uint64_t a, uint64_t b, uint32_t id, bool acc) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(d), "l"(a), "l"(b), "r"(id), "r"((int)acc));
}
// D (TMEM) (+)= A (TMEM) * B (shared)^T
__device__ __forceinline__ void mma_ts(uint32_t d, uint32_t a, uint64_t b, uint32_t id, bool acc) {
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n"
                 :: "r"(d), "r"(a), "l"(b), "r"(id), "r"((int)acc));
}
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(smem_u32(mbar)));
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// One poll: true once the phase with the given parity has completed.
__device__ __forceinline__ bool mbar_test(uint64_t* mbar, uint32_t parity) {
    uint32_t done = 0;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(smem_u32(mbar)), "r"(parity) : "memory");
    return done != 0;
}
// One non-blocking poll (mbarrier.test_wait): true once the phase with the given parity has
// completed.  try_wait above may itself wait for a system-dependent time.
__device__ __forceinline__ bool mbar_test_now(uint64_t* mbar, uint32_t parity) {
    uint32_t done = 0;
    asm volatile("{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(smem_u32(mbar)), "r"(parity) : "memory");
    return done != 0;
}
// One poll that may suspend the thread until the phase completes or about `hint_ns`
// nanoseconds have passed (a sleeping waiter takes no issue slots).
__device__ __forceinline__ bool mbar_test_sleep(uint64_t* mbar, uint32_t parity, uint32_t hint_ns) {
    uint32_t done = 0;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(done) : "r"(smem_u32(mbar)), "r"(parity), "r"(hint_ns) : "memory");
    return done != 0;
}
// Waits for the phase with the given parity; gives up after `limit` polls and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, long limit) {
    for (long it = 0; it < limit; ++it)
        if (mbar_test(mbar, parity)) return true;
    return false;
}
// The same, also giving up (false) as soon as *abort is set; on running out of polls it sets
// *abort itself, so that every other waiter of the CTA gives up too.  With hint_ns > 0 each
// poll may sleep up to that long (the wait is then bounded by limit * hint_ns); with
// hint_ns == 0 the polls do not block (a limit of a few polls then runs out for sure).
__device__ __forceinline__ bool mbar_wait_or_abort(uint64_t* mbar, uint32_t parity, long limit, volatile int* abort,
                                                   uint32_t hint_ns = 0) {
    for (long it = 0; it < limit; ++it) {
        if (hint_ns ? mbar_test_sleep(mbar, parity, hint_ns) : mbar_test_now(mbar, parity)) return true;
        if (*abort) return false;
    }
    *abort = 1;
    return false;
}
// Arrival of the calling thread (release semantics: its earlier shared-memory writes are
// visible to threads that observe the phase complete).
__device__ __forceinline__ void mbar_arrive(uint64_t* mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(mbar)) : "memory");
}

// TMEM allocation by one full warp; the base address is written to *slot (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(smem_u32(slot)), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t base, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(base), "r"(ncols));
}

// TMEM loads / stores of this thread's lane, `N` consecutive FP32 columns
__device__ __forceinline__ void ld1(uint32_t a, float& x) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=f"(x) : "r"(a));
}
__device__ __forceinline__ void ld2(uint32_t a, float* x) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=f"(x[0]), "=f"(x[1]) : "r"(a));
}
__device__ __forceinline__ void ld8(uint32_t a, float* x) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(x[0]), "=f"(x[1]), "=f"(x[2]), "=f"(x[3]), "=f"(x[4]), "=f"(x[5]), "=f"(x[6]), "=f"(x[7])
                 : "r"(a));
}
__device__ __forceinline__ void ld4(uint32_t a, float* x) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(x[0]), "=f"(x[1]), "=f"(x[2]), "=f"(x[3]) : "r"(a));
}
__device__ __forceinline__ void ld16(uint32_t a, float* x) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=f"(x[0]), "=f"(x[1]), "=f"(x[2]), "=f"(x[3]), "=f"(x[4]), "=f"(x[5]), "=f"(x[6]), "=f"(x[7]),
                   "=f"(x[8]), "=f"(x[9]), "=f"(x[10]), "=f"(x[11]), "=f"(x[12]), "=f"(x[13]), "=f"(x[14]), "=f"(x[15])
                 : "r"(a));
}
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void st1(uint32_t a, float x) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x1.b32 [%0], {%1};" :: "r"(a), "f"(x));
}
__device__ __forceinline__ void st2(uint32_t a, const float* x) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x2.b32 [%0], {%1,%2};" :: "r"(a), "f"(x[0]), "f"(x[1]));
}
__device__ __forceinline__ void st8(uint32_t a, const float* x) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                 :: "r"(a), "f"(x[0]), "f"(x[1]), "f"(x[2]), "f"(x[3]), "f"(x[4]), "f"(x[5]), "f"(x[6]), "f"(x[7]));
}
__device__ __forceinline__ void st4(uint32_t a, const float* x) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};"
                 :: "r"(a), "f"(x[0]), "f"(x[1]), "f"(x[2]), "f"(x[3]));
}
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// N consecutive columns of this thread's lane (N known at compile time), in x8/x4/x2/x1 pieces
template <int N>
__device__ __forceinline__ void ldn(uint32_t a, float* x) {
    if constexpr (N >= 8) { ld8(a, x); ldn<N - 8>(a + 8, x + 8); }
    else if constexpr (N >= 4) { ld4(a, x); ldn<N - 4>(a + 4, x + 4); }
    else if constexpr (N >= 2) { ld2(a, x); ldn<N - 2>(a + 2, x + 2); }
    else if constexpr (N == 1) { ld1(a, x[0]); }
}
template <int N>
__device__ __forceinline__ void stn(uint32_t a, const float* x) {
    if constexpr (N >= 8) { st8(a, x); stn<N - 8>(a + 8, x + 8); }
    else if constexpr (N >= 4) { st4(a, x); stn<N - 4>(a + 4, x + 4); }
    else if constexpr (N >= 2) { st2(a, x); stn<N - 2>(a + 2, x + 2); }
    else if constexpr (N == 1) { st1(a, x[0]); }
}

// Bulk (TMA) copy of `bytes` contiguous bytes global -> shared, completing on `mbar` as a
// transaction count; the issuing thread first arms the barrier with the expected bytes.
__device__ __forceinline__ void mbar_expect_tx(uint64_t* mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(mbar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(mbar)) : "memory");
}

// hint: bring [p, p + bytes) into L2 (bulk async prefetch; 16-byte aligned, bytes % 16 == 0)
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(bytes) : "memory");
}

// 3xTF32 split: x = hi + lo with hi, lo both TF32 (low 13 mantissa bits zero)
__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
__device__ __forceinline__ void split3(float x, float& hi, float& lo) {
    hi = tf32_hi(x);
    lo = tf32_hi(x - hi);
}

}  // namespace tc
}  // namespace dgx
