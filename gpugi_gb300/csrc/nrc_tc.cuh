// Fifth-generation tensor-core (tcgen05) building blocks of the radiance
// cache's MLP kernels: shared-memory matrix descriptors, the instruction
// descriptor of kind::f16, MMA issue and commit, bounded mbarrier waits and
// tensor-memory (TMEM) loads. Inline PTX for sm_100-class GPUs.
//
// Operands live in shared memory in the no-swizzle core-matrix layout: a core
// matrix is 8 rows of 16 bytes (8 halves) stored contiguously (128 B). For an
// operand whose contiguous dimension is c and strided dimension s, element
// (s, c) sits at (s / 8) * strideS + (c / 8) * strideC + (s % 8) * 16 +
// (c % 8) * 2 bytes. A descriptor gives the stride between core matrices
// along K ("leading byte offset") and along M or N ("stride byte offset"),
// whichever of the two dimensions is the contiguous one (K-major or
// MN-major operand, bits 15 / 16 of the instruction descriptor).
#pragma once
#include <cstdint>

#include "common.cuh"

namespace gpugi {
namespace nrc {
namespace tc {

GPUGI_D uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (no swizzle, descriptor version 1).
GPUGI_D uint64_t desc(uint32_t addr, uint32_t kStride, uint32_t mnStride) {
    uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((kStride >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((mnStride >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of tcgen05.mma kind::f16: f16 A and B, f32 D, dense.
GPUGI_HD constexpr uint32_t idesc(int M, int N, bool aMN, bool bMN) {
    return (1u << 4) | ((aMN ? 1u : 0u) << 15) | ((bMN ? 1u : 0u) << 16) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

// D (TMEM) = A * B (+ D when accumulate), issued by one thread.
GPUGI_D void mma(uint32_t dTmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dTmem),
        "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

// The mbarrier completes a phase once every MMA this thread issued before is done.
GPUGI_D void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

GPUGI_D void bar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// The global timer in nanoseconds.
GPUGI_D uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase `parity` of an mbarrier, at most limitNs nanoseconds
// of the global timer (and at most 2^24 polls, should the timer not
// advance); false when the wait ran out.
GPUGI_D bool bar_wait(uint64_t* bar, uint32_t parity, uint64_t limitNs) {
    const uint32_t a = smem_addr(bar);
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t it = 0; it < (1u << 24); ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 255u && globaltimer_ns() - t0 > limitNs) return false;
    }
    return false;
}

GPUGI_D void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
GPUGI_D void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory stores become visible to the tensor cores.
GPUGI_D void fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Allocation by one whole warp; the column base lands in *slot.
GPUGI_D void tmem_alloc(uint32_t* slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
GPUGI_D void tmem_free(uint32_t base, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(cols));
}

// 16 consecutive 32-bit columns of this thread's TMEM lane (warp w reads
// lanes 32 (w % 4) .. + 31); complete after ld_wait.
GPUGI_D void ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
GPUGI_D void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Byte offset of element (s, c) of a core-matrix layout (c contiguous).
GPUGI_HD constexpr uint32_t cm_off(uint32_t s, uint32_t c, uint32_t strideS, uint32_t strideC) {
    return (s / 8) * strideS + (c / 8) * strideC + (s % 8) * 16 + (c % 8) * 2;
}

}  // namespace tc
}  // namespace nrc
}  // namespace gpugi
