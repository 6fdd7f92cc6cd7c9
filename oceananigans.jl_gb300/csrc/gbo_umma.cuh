// gbo_umma.cuh -- fifth-generation tensor-core (tcgen05) primitives for sm_100 / sm_103.
//
// One elected thread of a CTA issues tcgen05.mma with both operands in shared memory
// and the FP32 accumulator in tensor memory (TMEM); the CTA's warps read the
// accumulator back with tcgen05.ld.  Operands use the canonical K-major layout without
// swizzle: the operand is a grid of 8-row × 16-byte core matrices (8 rows of 8 BF16
// values of consecutive k, 128 contiguous bytes); LBO is the byte distance between the
// two core matrices of one MMA's K = 16 (k 0-7 and 8-15), SBO the distance between
// consecutive groups of 8 rows.  Completion is signalled through an mbarrier that
// tcgen05.commit arrives on; every wait on it is bounded and reports a timeout instead
// of spinning forever.
#pragma once
#include <cstdint>

namespace umma {

GBO_D uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, LBO and SBO in 16-byte units, the
// descriptor version of tcgen05 (bits 46-47 = 1), base offset 0, no swizzle (bits 61-63 = 0).
GBO_D uint64_t sdesc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D, both K-major, M × N:
// D format bits 4-5 = 1 (F32), A format bits 7-9 = 1 (BF16), B format bits 10-12 = 1,
// N >> 3 at bits 17-22, M >> 4 at bits 24-28.
GBO_HD constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// TMEM columns (a power of two, at least 32) allocated by one whole warp; the address
// is written to *slot in shared memory.  The same warp frees them.
GBO_D void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::);
}
GBO_D void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
GBO_D void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::); }
GBO_D void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::); }
// generic-proxy writes to shared memory (plain stores, cp.async) made visible to the
// tensor cores, which read operands through the async proxy
GBO_D void fence_smem_to_async() { asm volatile("fence.proxy.async.shared::cta;" ::); }

// D (+)= A B^T: one MMA of M × N × 16
GBO_D void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, bool accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate));
}
// the mbarrier arrives once every MMA this thread issued before has completed
GBO_D void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar)));
}

GBO_D void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::);
}
// Wait for the phase with the given parity to complete; false after `limit` polls.
GBO_D bool mbar_wait(uint64_t* mbar, uint32_t parity, int limit) {
    uint32_t done = 0;
    for (int it = 0; it < limit && !done; ++it)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(smem_addr(mbar)), "r"(parity));
    return done != 0;
}

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane: warp w of the CTA
// reads lanes 32 (w mod 4) .. + 31 (row m = 32 (w mod 4) + lane of an M = 128 tile).
GBO_D void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::);
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

}  // namespace umma
