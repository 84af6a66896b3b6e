// Tensor-core (tcgen05, kind::tf32) form of the sigma-accumulation phase of
// H_eff*psi on sm_103a, split-TF32 x3 with FP32 accumulation in TMEM.
//
// One CTA (4 warps) owns one 128-row x N-column tile of a sigma region
// (N <= 256, multiple of 16).  The tile's GEMM1 contributions
// alpha * op(L) (rows x k1) * W (k1 x cols) are concatenated along K and
// packed into stages of kTcStageK = 16 columns.  Per stage, all 128 threads
// stage the A slab (128 x 16, alpha folded in, operators (FP32 copy) split
// into a TF32 "hi" part and a TF32 "lo" remainder) and the B slab (N x 16
// from W)
// into shared memory in the canonical no-swizzle K-major layout (8-row x
// 16-byte core matrices, LBO = 128 B along K, SBO = 512 B along M/N), then
// one elected thread issues, per K = 8 half, the three products
// hi*hi + hi*lo + lo*hi as tcgen05.mma into one TMEM accumulator
// (128 lanes x N fp32 columns) and commits them to the stage buffer's
// mbarrier.  Two stage buffers alternate so staging overlaps the MMAs.
// The epilogue reads TMEM with tcgen05.ld (each warp its 32-lane quarter)
// and adds scale * D into sigma (FP64) for the cells the region owns.
//
// The operands are gathered from scattered operator blocks of irregular
// shape and stride (transposed or not, arbitrary double offsets), so they
// are staged with plain loads rather than TMA (a TMA copy needs 16-byte
// aligned starts and fixed boxes, which these blocks do not have).
//
// Every mbarrier wait is bounded: on timeout the kernel sets *err, waits
// (bounded) for its outstanding MMAs, frees its TMEM and returns.
#include "b2g_internal.h"

namespace b2g {

namespace {

constexpr int kThreads = 128;
constexpr int kMaxN = 256;
constexpr uint32_t kABytes = 128 * kTcStageK * 4;      // 8 KB per split part
constexpr uint32_t kBBytes = kMaxN * kTcStageK * 4;    // 16 KB per split part
constexpr uint32_t kBufBytes = 2 * kABytes + 2 * kBBytes;  // hi+lo of A and B: 48 KB
constexpr uint32_t kSmemBytes = 2 * kBufBytes + 2048;  // two buffers + barriers + alignment slack
constexpr uint32_t kSBO = (kTcStageK / 4) * 128;       // bytes between 8-row groups
constexpr uint32_t kLBO = 128;                         // bytes between K-adjacent core matrices
constexpr long long kSpinLimit = 1ll << 22;  // an MMA group completes in microseconds

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm volatile("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// byte offset of element (row, k) in a canonical no-swizzle K-major tile
__device__ __forceinline__ uint32_t kmajor_off(int row, int k) {
    return (uint32_t)((row >> 3) * kSBO + (k >> 2) * kLBO + (row & 7) * 16 + (k & 3) * 4);
}

// tcgen05 shared-memory matrix descriptor: no swizzle, K-major
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(kLBO >> 4) << 16;
    d |= (uint64_t)(kSBO >> 4) << 32;
    d |= (uint64_t)1 << 46;  // fixed constant 0b001 of the tcgen05 descriptor
    return d;                // base offset 0, swizzle mode 0 (none)
}

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major, M = 128
__device__ __forceinline__ uint32_t make_idesc(int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(dtmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// bounded wait for phase `parity` of an mbarrier; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (long long it = 0; it < kSpinLimit; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
        if (done)
            return true;
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 consecutive fp32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
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
__device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
    hi = to_tf32(x);
    lo = to_tf32(x - __uint_as_float(hi));
}

// per-stage copy of the segments and contribution fields staging needs
struct StageSeg {
    const float *A;   // operator block of the contribution (FP32 copy of the blob)
    const float *W;   // work matrix of the contribution
    float alpha;
    int32_t row0, m1, lda1, ta1, col0, n1, kb, koff, kl;
};

__global__ void __launch_bounds__(kThreads, 1)
tc_phase2_kernel(const TcTask *__restrict__ tasks, const TcTile *__restrict__ tiles,
                 const TcSeg *__restrict__ segs, const Contrib *__restrict__ contribs,
                 const Region *__restrict__ regions, const WorkDesc *__restrict__ works,
                 const float *__restrict__ ops, const float *__restrict__ work,
                 double *__restrict__ sigma, float *__restrict__ part, double scale, int *err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *mbar = (uint64_t *)(smem + 2 * kBufBytes);      // [0], [1]: stage buffers
    uint32_t *tmem_slot = (uint32_t *)(smem + 2 * kBufBytes + 64);
    __shared__ StageSeg sseg[kTcStageK];
    __shared__ int8_t col_seg[kTcStageK];   // stage column -> sseg index (-1: zero column)
    __shared__ int8_t col_kk[kTcStageK];    // stage column -> k offset inside the segment
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const TcTask tk = tasks[blockIdx.x];
    const TcTile tl = tiles[tk.tile];
    const Region rg = regions[tl.g];

    if (tid == 0) {
        mbar_init(smem_u32(&mbar[0]), 1);
        mbar_init(smem_u32(&mbar[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(tmem_slot)), "r"(kMaxN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = make_idesc(tl.n);
    int issued = 0;      // stages whose MMAs were committed
    int64_t sp = tk.sb;  // segment cursor (segments are ordered by stage)
    for (int ls = 0; ls < tk.n_stages; ls++) {
        const int st = tk.st0 + ls;
        const int b = ls & 1;
        unsigned char *buf = smem + b * kBufBytes;
        // buffer b was last read by the MMAs of local stage ls-2 (CTA-uniform outcome)
        if (ls >= 2) {
            const int good = __syncthreads_and(
                mbar_wait(smem_u32(&mbar[b]), (uint32_t)(((ls >> 1) - 1) & 1)) ? 1 : 0);
            if (!good) {
                if (tid == 0)
                    atomicExch(err, 1);
                break;
            }
        }
        // ---- this stage's segment table
        if (tid < kTcStageK)
            col_seg[tid] = -1;
        __syncthreads();
        const int64_t si = sp + tid;
        const bool mine = tid < kTcStageK && si < tk.se && segs[si].stage == st;
        if (mine) {
            const TcSeg sg = segs[si];
            const Contrib c = contribs[sg.c];
            StageSeg x;
            x.A = ops + c.a1;
            x.W = work + works[c.u].woff;
            x.alpha = (float)c.alpha;
            x.row0 = c.row0, x.m1 = c.m1, x.lda1 = c.lda1, x.ta1 = c.ta1;
            x.col0 = c.col0, x.n1 = c.n1, x.kb = sg.kb, x.koff = sg.koff, x.kl = sg.kl;
            sseg[tid] = x;
            for (int kk = 0; kk < sg.kl; kk++)
                col_seg[sg.koff + kk] = (int8_t)tid, col_kk[sg.koff + kk] = (int8_t)kk;
        }
        sp += __syncthreads_count(mine ? 1 : 0);
        // ---- stage the A slab: thread tid owns tile row tid
        {
            const int row = tl.row0 + tid;
#pragma unroll
            for (int k4 = 0; k4 < kTcStageK / 4; k4++) {
                uint32_t h[4], l[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    h[j] = 0u, l[j] = 0u;
                    const int q = 4 * k4 + j, si2 = col_seg[q];
                    if (si2 >= 0) {
                        const StageSeg &x = sseg[si2];
                        const int ar = row - x.row0;
                        if (ar >= 0 && ar < x.m1) {
                            const int k = x.kb + col_kk[q];
                            const float a = x.alpha * (x.ta1 ? x.A[(uint64_t)k * x.lda1 + ar]
                                                             : x.A[(uint64_t)ar * x.lda1 + k]);
                            split_tf32(a, h[j], l[j]);
                        }
                    }
                }
                const uint32_t off = kmajor_off(tid, 4 * k4);
                *(uint4 *)(buf + off) = make_uint4(h[0], h[1], h[2], h[3]);
                *(uint4 *)(buf + kABytes + off) = make_uint4(l[0], l[1], l[2], l[3]);
            }
        }
        // ---- stage the B slab: B[n][k] = W(k, n); threads own columns tid, tid + 128
        for (int nn = tid; nn < tl.n; nn += kThreads) {
            const int col = tl.col0 + nn;
#pragma unroll
            for (int k4 = 0; k4 < kTcStageK / 4; k4++) {
                uint32_t h[4], l[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    h[j] = 0u, l[j] = 0u;
                    const int q = 4 * k4 + j, si2 = col_seg[q];
                    if (si2 >= 0) {
                        const StageSeg &x = sseg[si2];
                        const int wc = col - x.col0;
                        if (wc >= 0 && wc < x.n1) {
                            const float w = x.W[(uint64_t)(x.kb + col_kk[q]) * x.n1 + wc];
                            split_tf32(w, h[j], l[j]);
                        }
                    }
                }
                const uint32_t off = kmajor_off(nn, 4 * k4);
                *(uint4 *)(buf + 2 * kABytes + off) = make_uint4(h[0], h[1], h[2], h[3]);
                *(uint4 *)(buf + 2 * kABytes + kBBytes + off) = make_uint4(l[0], l[1], l[2], l[3]);
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t a_hi = smem_u32(buf), a_lo = a_hi + kABytes;
            const uint32_t b_hi = a_hi + 2 * kABytes, b_lo = b_hi + kBBytes;
#pragma unroll
            for (int h = 0; h < kTcStageK / 8; h++) {
                const uint32_t ko = h * 2 * kLBO;  // K = 8 = two core matrices
                const uint32_t acc0 = (ls > 0 || h > 0) ? 1u : 0u;
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_hi + ko), idesc, acc0);
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_lo + ko), idesc, 1u);
                mma_tf32(tmem, make_desc(a_lo + ko), make_desc(b_hi + ko), idesc, 1u);
            }
            mma_commit(smem_u32(&mbar[b]));
        }
        issued = ls + 1;
    }
    // wait for the last issued stage's MMAs (its commit covers all earlier ones)
    const int last = issued - 1;
    bool done = false;
    if (last >= 0) {
        const int b = last & 1;
        done = __syncthreads_and(mbar_wait(smem_u32(&mbar[b]), (uint32_t)((last >> 1) & 1)) ? 1 : 0) != 0;
        if (!done && tid == 0)
            atomicExch(err, 1);
    }
    tc_fence_after();
    if (done && issued == tk.n_stages) {
        // ---- epilogue: warp w holds TMEM lanes [32w, 32w + 32) = tile rows
        const int trow = warp * 32 + lane;
        const int row = tl.row0 + trow;
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
        float *prow = tl.part >= 0 ? part + tl.part + ((int64_t)tk.chunk * 128 + trow) * tl.n : nullptr;
        for (int c16 = 0; c16 < tl.n; c16 += 16) {
            float v[16];
            tmem_ld16(tbase + (uint32_t)c16, v);
            if (prow != nullptr) {
#pragma unroll
                for (int j = 0; j < 16; j += 4)
                    *(float4 *)(prow + c16 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            } else if (trow < tl.rows) {
                const uint64_t rowaddr = rg.base + (uint64_t)row * rg.ld;
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int col = tl.col0 + c16 + j;
                    const uint64_t a = rowaddr + (uint64_t)col;
                    if (col < rg.cols && a >= rg.lo && a < rg.hi)
                        sigma[a] += scale * (double)v[j];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kMaxN));
}

// split-K reduction: sigma += scale * sum over chunks (fixed order) of the partial tiles
__global__ void __launch_bounds__(256) tc_reduce_kernel(const int32_t *__restrict__ multi,
                                                        const TcTile *__restrict__ tiles,
                                                        const Region *__restrict__ regions,
                                                        const float *__restrict__ part,
                                                        double *__restrict__ sigma, double scale) {
    const TcTile tl = tiles[multi[blockIdx.x]];
    const Region rg = regions[tl.g];
    const int64_t plane = (int64_t)128 * tl.n;
    for (int e = threadIdx.x; e < tl.rows * tl.n; e += blockDim.x) {
        const int r = e / tl.n, cc = e % tl.n;
        const int col = tl.col0 + cc;
        const uint64_t a = rg.base + (uint64_t)(tl.row0 + r) * rg.ld + (uint64_t)col;
        if (col >= rg.cols || a < rg.lo || a >= rg.hi)
            continue;
        double s = 0.0;
        const float *p = part + tl.part + (int64_t)r * tl.n + cc;
        for (int ch = 0; ch < tl.n_chunks; ch++)
            s += (double)p[ch * plane];
        sigma[a] += scale * s;
    }
}

} // namespace

cudaError_t launch_tc_phase2(const DevicePlan &p, const float *ops, const float *work,
                             double *sigma, double scale, int *err, cudaStream_t s) {
    if (p.n_tct == 0)
        return cudaSuccess;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(tc_phase2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kSmemBytes);
        if (e != cudaSuccess)
            return e;
        attr_set = true;
    }
    tc_phase2_kernel<<<(unsigned)p.n_tct, kThreads, kSmemBytes, s>>>(
        p.tct, p.tctile, p.tcs, p.contribs, p.regions, p.works, ops, work, sigma, p.tc_part, scale, err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || p.n_tc_multi == 0)
        return e;
    tc_reduce_kernel<<<(unsigned)p.n_tc_multi, 256, 0, s>>>(p.tc_multi, p.tctile, p.regions, p.tc_part,
                                                            sigma, scale);
    return cudaGetLastError();
}

} // namespace b2g
