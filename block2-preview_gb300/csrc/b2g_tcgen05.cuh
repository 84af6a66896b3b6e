// tcgen05 / mbarrier / bulk-copy helpers shared by the tensor-core kernels
// (inline PTX for sm_103a).  Shared-memory operand tiles use the canonical
// no-swizzle K-major layout: 8-row x 16-byte core matrices, LBO = 128 B
// between K-adjacent core matrices, SBO = 512 B between 8-row groups (a
// 16-column FP32/TF32 K slab).
#pragma once

#include <stdint.h>

namespace b2g {
namespace tcg {

constexpr uint32_t kSBO = 512;                          // bytes between 8-row groups (K slab of 16)
constexpr uint32_t kLBO = 128;                         // bytes between K-adjacent core matrices
constexpr long long kSpinLimit = 1ll << 23;            // bounded waits (tries, mostly 256 ns apart)

static __device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

static __device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm volatile("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// byte offset of element (row, k) in a canonical no-swizzle K-major tile
static __device__ __forceinline__ uint32_t kmajor_off(int row, int k) {
    return (uint32_t)((row >> 3) * kSBO + (k >> 2) * kLBO + (row & 7) * 16 + (k & 3) * 4);
}

// tcgen05 shared-memory matrix descriptor: no swizzle, K-major
static __device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(kLBO >> 4) << 16;
    d |= (uint64_t)(kSBO >> 4) << 32;
    d |= (uint64_t)1 << 46;  // fixed constant 0b001 of the tcgen05 descriptor
    return d;                // base offset 0, swizzle mode 0 (none)
}

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major, M = 128
static __device__ __forceinline__ uint32_t make_idesc(int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

static __device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

static __device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(mbar) : "memory");
}

static __device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// bounded wait for phase `parity` of an mbarrier; false on timeout.  After a
// few immediate tries the waiting thread backs off with __nanosleep (32 ns
// doubling to 256 ns), so waiting warps leave the issue slots to the warps
// doing the work; at most kSpinLimit tries (about two seconds).
static __device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    uint32_t ns = 32;
    for (long long it = 0; it < kSpinLimit; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
        if (done)
            return true;
        if (it >= 4) {
            __nanosleep(ns);
            ns = ns < 256 ? 2 * ns : 256;
        }
    }
    return false;
}

static __device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

static __device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
static __device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 consecutive fp32 columns of this thread's TMEM lane
static __device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++)
        v[i] = __uint_as_float(r[i]);
}

// split x into TF32 hi + TF32 lo (x - hi, exact in FP32), raw fp32 bit patterns;
// FP32 arithmetic only (FP64 work would run on GB300's narrow FP64 pipe)
static __device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
    hi = to_tf32(x);
    lo = to_tf32(x - __uint_as_float(hi));
}

static __device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}


// mbarrier arrive that also announces `bytes` of asynchronous transfers
static __device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
                 : "memory");
}

// bulk copy (TMA, no tensor map) of `bytes` contiguous bytes global -> shared,
// completing on `mbar`; both addresses 16-byte aligned, bytes a multiple of 16
static __device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                                uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "l"(src), "r"(bytes), "r"(mbar) : "memory");
}

} // namespace tcg
} // namespace b2g
