// umma.cuh — fifth-generation tensor-core (tcgen05) building blocks for sm_103a, written as inline PTX: tensor-memory
// allocation, shared-memory matrix descriptors, the FP16 MMA with FP32 accumulation in tensor memory, completion
// through an mbarrier (bounded wait) and tensor-memory loads.
//
// Shared-memory operands use the canonical K-major layout without swizzling: a matrix of R rows and K columns (FP16)
// is cut into core matrices of 8 rows x 8 columns (8 rows of 16 bytes, 128 contiguous bytes); core matrices that
// follow each other along K are kUmmaLbo bytes apart, groups of 8 rows kUmmaSbo bytes apart. With K = 64 an 8-row group
// is 8 core matrices = 1 KB, so element (r, k) sits at (r / 8) * 1024 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2.
// One MMA consumes K = 16, two core matrices along K; the next K step starts 256 bytes further.
#pragma once

#include <cstdint>

#include "common.cuh"

namespace vkrt {

constexpr uint32_t kUmmaLbo = 128u;   // bytes between core matrices along K
constexpr uint32_t kUmmaSbo = 1024u;  // bytes between 8-row groups (K = 64)

// byte offset of element (r, k) of a K = 64 operand in the canonical K-major layout
VKRT_DEV uint32_t ummaOffset(uint32_t r, uint32_t k) {
    return (r >> 3) * kUmmaSbo + (k >> 3) * kUmmaLbo + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Shared-memory matrix descriptor: start address, leading (K) and stride (row-group) byte offsets, each >> 4;
// descriptor version 1 (bits 46-47); no swizzling (layout type 0, bits 61-63); base offset 0.
VKRT_DEV uint64_t ummaSmemDesc(uint32_t smemAddr) {
    return uint64_t((smemAddr >> 4) & 0x3FFFu) | (uint64_t((kUmmaLbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((kUmmaSbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1u) << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), FP16 A and B (bits 7-9, 10-12 = 0), both
// operands K-major (bits 15, 16 = 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28.
VKRT_HD constexpr uint32_t ummaIdescF16(uint32_t m, uint32_t n) {
    return (1u << 4) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

VKRT_DEV uint32_t smemAddr(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

// Tensor-memory columns: allocated by one whole warp, the base address written to shared memory `slot`.
VKRT_DEV void tmemAlloc(uint32_t* slot, uint32_t columns) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(slot)),
                 "r"(columns));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
}
VKRT_DEV void tmemFree(uint32_t tmem, uint32_t columns) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(columns));
}

VKRT_DEV void tcgenFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
VKRT_DEV void tcgenFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// generic-proxy writes to shared memory made visible to the tensor core's reads of the same memory
VKRT_DEV void fenceProxyAsyncShared() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

VKRT_DEV void mbarInit(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smemAddr(bar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// D (tensor memory) = A B^T (+ D when accumulate), A and B K-major FP16 in shared memory; issued by one thread.
VKRT_DEV void ummaF16(uint32_t tmemD, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmemD),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// The mbarrier's phase completes once every MMA this thread issued before has finished.
VKRT_DEV void ummaCommit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smemAddr(bar))
                 : "memory");
}

// Waits for phase `parity` of the mbarrier, at most `limit` polls; false when it did not complete.
VKRT_DEV bool mbarWait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    const uint32_t a = smemAddr(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 16 consecutive FP32 columns of this thread's tensor-memory lane (a warp reads lanes 32 w .. 32 w + 31 of the
// address it passes); valid after tmemLoadWait.
VKRT_DEV void tmemLoad16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
VKRT_DEV void tmemLoadWait() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

}  // namespace vkrt
