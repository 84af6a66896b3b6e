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

constexpr int kThreads = 256;                          // 8 warps
constexpr int kProducers = 7;                          // warps 0..6 stage operands
constexpr int kMmaWarp = 7;                            // lane 0 of warp 7 issues the MMAs
constexpr int kMaxN = 256;
constexpr int kMaxRing = 8;
constexpr uint32_t kABytes = 128 * kTcStageK * 4;      // 8 KB per split part of A
constexpr uint32_t kRingBytes = 192 * 1024;            // ring of stage slots
constexpr uint32_t kSegBytes = kTcMaxSegs * sizeof(TcSeg);
constexpr uint32_t kSmemBytes = kRingBytes + kSegBytes + 4 * (kTcMaxSegs + 2) + 256 + 1024;
constexpr uint32_t kSBO = (kTcStageK / 4) * 128;       // bytes between 8-row groups
constexpr uint32_t kLBO = 128;                         // bytes between K-adjacent core matrices
constexpr long long kSpinLimit = 1ll << 24;            // bounded waits (a stage takes microseconds)

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

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// One CTA per chunk (a K range of one 128 x N tile).  Warps 0..6 are
// producers: stage s is filled by warp s % 7 into ring slot s % R (A slab
// 128 x 16 and B slab N x 16, TF32 hi/lo each), then released to the MMA
// thread through full[slot].  Lane 0 of warp 7 waits on full[slot], issues
// the 3 x 2 MMAs of the stage into the TMEM accumulator and commits them to
// empty[slot], which frees the slot for stage s + R.  No CTA-wide barrier is
// taken in the main loop, so several stages' global loads are in flight at
// once.  All 8 warps drain TMEM at the end (warp w: lanes of quarter w % 4,
// every other 16-column chunk).
__global__ void __launch_bounds__(kThreads, 1)
tc_phase2_kernel(const TcTask *__restrict__ tasks, const TcTile *__restrict__ tiles,
                 const TcSeg *__restrict__ segs, const Region *__restrict__ regions,
                 const float *__restrict__ ops, const float *__restrict__ work,
                 double *__restrict__ sigma, float *__restrict__ part, double scale, int *err,
                 RootStrides rs) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    work += blockIdx.y * rs.work;
    sigma += blockIdx.y * rs.sigma;
    part += blockIdx.y * rs.part;
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    TcSeg *sseg = (TcSeg *)(smem + kRingBytes);
    int32_t *stage_start = (int32_t *)(smem + kRingBytes + kSegBytes);
    uint64_t *full = (uint64_t *)(smem + kRingBytes + kSegBytes + 4 * (kTcMaxSegs + 2));
    uint64_t *empty = full + kMaxRing;
    uint64_t *done = empty + kMaxRing;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    int *abort_flag = (int *)(tmem_slot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const TcTask tk = tasks[blockIdx.x];
    const TcTile tl = tiles[tk.tile];
    const Region rg = regions[tl.g];
    const int nseg = (int)(tk.se - tk.sb);
    const uint32_t slot_bytes = (2 * kABytes + (uint32_t)tl.n * kTcStageK * 8 + 1023) & ~1023u;
    // P producer warps, each owning D ring slots (slot = p + P * (j % D) for its
    // j-th stage): every slot is then filled by one warp in order, so no waiter
    // is ever two mbarrier phases behind (parity waits would alias there)
    const int Rmax = min(kMaxRing, (int)(kRingBytes / slot_bytes));
    const int P = min(kProducers, Rmax), D = Rmax / P, R = P * D;

    // ---- setup: segment table, stage starts, barriers, TMEM
    for (int i = tid; i < nseg; i += kThreads)
        sseg[i] = segs[tk.sb + i];
    if (tid == 0) {
        for (int i = 0; i < R; i++) {
            mbar_init(smem_u32(&full[i]), 1);
            mbar_init(smem_u32(&empty[i]), 1);
        }
        mbar_init(smem_u32(done), 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(tmem_slot)), "r"(kMaxN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    __syncthreads();
    // stage_start[j] = first local segment of stage st0 + j (segments ordered by stage)
    for (int i = tid; i < nseg; i += kThreads) {
        const int j = sseg[i].stage - tk.st0;
        if (i == 0 || sseg[i - 1].stage != sseg[i].stage)
            stage_start[j] = i;
    }
    if (tid == 0)
        stage_start[tk.n_stages] = nseg;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp < P) {
        // ---------------- producers
        for (int ls = warp, j = 0; ls < tk.n_stages; ls += P, j++) {
            const int slot = warp + P * (j % D), use = j / D;
            unsigned char *buf = smem + (uint32_t)slot * slot_bytes;
            if (use >= 1) {
                bool ok = false;
                if (lane == 0)
                    ok = mbar_wait(smem_u32(&empty[slot]), (uint32_t)((use - 1) & 1));
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) {
                    if (lane == 0) {
                        atomicExch(err, 1);
                        atomicExch(abort_flag, 1);
                    }
                    break;
                }
            }
            // column map of this stage: lanes 0..15 find their column's segment
            const int s0 = stage_start[ls], s1 = stage_start[ls + 1];
            int my_seg = -1, my_kk = 0;
            if (lane < kTcStageK)
                for (int q = s0; q < s1; q++) {
                    const int ko = sseg[q].koff;
                    if (lane >= ko && lane < ko + sseg[q].kl) {
                        my_seg = q, my_kk = lane - ko;
                        break;
                    }
                }
            // ---- A slab: lane owns rows lane + 32 i (i < 4), all 16 columns
            float av[4][kTcStageK];
#pragma unroll
            for (int q = 0; q < kTcStageK; q++) {
                const int sq = __shfl_sync(0xffffffffu, my_seg, q);
                const int kk = __shfl_sync(0xffffffffu, my_kk, q);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    float v = 0.f;
                    if (sq >= 0) {
                        const TcSeg &x = sseg[sq];
                        const int ar = tl.row0 + lane + 32 * i - x.row0;
                        if (ar >= 0 && ar < x.m1) {
                            const int k = x.kb + kk;
                            v = x.alpha * __ldg(ops + x.a + (x.ta1 ? (uint64_t)k * x.lda1 + ar
                                                                   : (uint64_t)ar * x.lda1 + k));
                        }
                    }
                    av[i][q] = v;
                }
            }
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int row = lane + 32 * i;
#pragma unroll
                for (int k4 = 0; k4 < kTcStageK / 4; k4++) {
                    uint32_t h[4], l[4];
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        split_tf32(av[i][4 * k4 + j], h[j], l[j]);
                    const uint32_t off = kmajor_off(row, 4 * k4);
                    *(uint4 *)(buf + off) = make_uint4(h[0], h[1], h[2], h[3]);
                    *(uint4 *)(buf + kABytes + off) = make_uint4(l[0], l[1], l[2], l[3]);
                }
            }
            // ---- B slab: lane owns tile columns lane + 32 j, all 16 k
            const uint32_t b_hi = 2 * kABytes, b_lo = b_hi + (uint32_t)tl.n * kTcStageK * 4;
            for (int jb = 0; jb < tl.n; jb += 128) {
                float bv[4][kTcStageK];
#pragma unroll
                for (int q = 0; q < kTcStageK; q++) {
                    const int sq = __shfl_sync(0xffffffffu, my_seg, q);
                    const int kk = __shfl_sync(0xffffffffu, my_kk, q);
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        float v = 0.f;
                        const int nn = jb + lane + 32 * j;
                        if (sq >= 0 && nn < tl.n) {
                            const TcSeg &x = sseg[sq];
                            const int wc = tl.col0 + nn - x.col0;
                            if (wc >= 0 && wc < x.n1)
                                v = __ldg(work + x.w + (uint64_t)(x.kb + kk) * x.n1 + wc);
                        }
                        bv[j][q] = v;
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int nn = jb + lane + 32 * j;
                    if (nn >= tl.n)
                        continue;
#pragma unroll
                    for (int k4 = 0; k4 < kTcStageK / 4; k4++) {
                        uint32_t h[4], l[4];
#pragma unroll
                        for (int jj = 0; jj < 4; jj++)
                            split_tf32(bv[j][4 * k4 + jj], h[jj], l[jj]);
                        const uint32_t off = kmajor_off(nn, 4 * k4);
                        *(uint4 *)(buf + b_hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
                        *(uint4 *)(buf + b_lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
                    }
                }
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(smem_u32(&full[slot]));
        }
    } else if (warp == kMmaWarp && lane == 0) {
        // ---------------- MMA issuer
        const uint32_t idesc = make_idesc(tl.n);
        for (int ls = 0; ls < tk.n_stages; ls++) {
            const int jj = ls / P, slot = ls % P + P * (jj % D), use = jj / D;
            if (!mbar_wait(smem_u32(&full[slot]), (uint32_t)(use & 1))) {
                atomicExch(err, 1);
                atomicExch(abort_flag, 1);
                break;
            }
            tc_fence_after();
            const uint32_t a_hi = smem_u32(smem + (uint32_t)slot * slot_bytes), a_lo = a_hi + kABytes;
            const uint32_t b_hi = a_hi + 2 * kABytes, b_lo = b_hi + (uint32_t)tl.n * kTcStageK * 4;
#pragma unroll
            for (int h = 0; h < kTcStageK / 8; h++) {
                const uint32_t ko = h * 2 * kLBO;  // K = 8 = two core matrices
                const uint32_t acc0 = (ls > 0 || h > 0) ? 1u : 0u;
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_hi + ko), idesc, acc0);
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_lo + ko), idesc, 1u);
                mma_tf32(tmem, make_desc(a_lo + ko), make_desc(b_hi + ko), idesc, 1u);
            }
            mma_commit(smem_u32(&empty[slot]));
        }
        mma_commit(smem_u32(done));  // tracks every MMA issued above
    }
    // ---- epilogue
    __syncwarp();
    const int good = __syncthreads_and(mbar_wait(smem_u32(done), 0u) ? 1 : 0);
    tc_fence_after();
    if (!good && tid == 0)
        atomicExch(err, 1);
    if (good && *abort_flag == 0) {
        const int q4 = warp & 3, half = warp >> 2;
        const int trow = q4 * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(q4 * 32) << 16);
        for (int c16 = half * 16; c16 < tl.n; c16 += 32) {
            float v[16];
            tmem_ld16(tbase + (uint32_t)c16, v);
            if (trow >= tl.rows)
                continue;
            if (tl.part >= 0) {
                float *prow = part + tl.part + ((int64_t)tk.chunk * tl.rows + trow) * tl.n + c16;
#pragma unroll
                for (int j = 0; j < 16; j += 4)
                    *(float4 *)(prow + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            } else {
                const uint64_t rowaddr = rg.base + (uint64_t)(tl.row0 + trow) * rg.ld;
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

// ---------------------------------------------------------------------------
// Phase 1 (GEMM0) on tensor cores: one CTA per Tc1Tile, D (128 x n) =
// stacked psi rows (128 x k0) * op(R) (k0 x n), same TF32 x3 split, same
// producer / single-thread-MMA ring as phase 2 (smaller ring: two CTAs per
// SM), epilogue writes the FP32 work rows.
constexpr uint32_t kRing1Bytes = 96 * 1024;
constexpr uint32_t kSmem1Bytes = kRing1Bytes + 128 * sizeof(Tc1Row) + 256 + 1024;

__global__ void __launch_bounds__(kThreads, 1)
tc_phase1_kernel(const Tc1Tile *__restrict__ tiles, const Tc1Row *__restrict__ rowtab,
                 const float *__restrict__ ops, const float *__restrict__ psi,
                 float *__restrict__ work, int *err, RootStrides rs) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    psi += blockIdx.y * rs.psi;
    work += blockIdx.y * rs.work;
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    Tc1Row *srow = (Tc1Row *)(smem + kRing1Bytes);
    uint64_t *full = (uint64_t *)(smem + kRing1Bytes + 128 * sizeof(Tc1Row));
    uint64_t *empty = full + kMaxRing;
    uint64_t *done = empty + kMaxRing;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    int *abort_flag = (int *)(tmem_slot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const Tc1Tile tl = tiles[blockIdx.x];
    const int n_stages = (tl.k0 + kTcStageK - 1) / kTcStageK;
    const uint32_t slot_bytes = (2 * kABytes + (uint32_t)tl.n * kTcStageK * 8 + 1023) & ~1023u;
    const int Rmax = min(kMaxRing, (int)(kRing1Bytes / slot_bytes));
    const int P = min(kProducers, Rmax), D = Rmax / P, R = P * D;
    const float *Rm = ops + tl.b0;

    for (int i = tid; i < tl.rows; i += kThreads)
        srow[i] = rowtab[tl.rb + i];
    if (tid == 0) {
        for (int i = 0; i < R; i++) {
            mbar_init(smem_u32(&full[i]), 1);
            mbar_init(smem_u32(&empty[i]), 1);
        }
        mbar_init(smem_u32(done), 1);
        *abort_flag = 0;
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

    if (warp < P) {
        for (int ls = warp, j = 0; ls < n_stages; ls += P, j++) {
            const int slot = warp + P * (j % D), use = j / D;
            unsigned char *buf = smem + (uint32_t)slot * slot_bytes;
            if (use >= 1) {
                bool ok = false;
                if (lane == 0)
                    ok = mbar_wait(smem_u32(&empty[slot]), (uint32_t)((use - 1) & 1));
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) {
                    if (lane == 0) {
                        atomicExch(err, 1);
                        atomicExch(abort_flag, 1);
                    }
                    break;
                }
            }
            const int k0 = ls * kTcStageK;
            // A: stacked psi rows lane + 32 i
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int row = lane + 32 * i;
                float av[kTcStageK];
                const bool live = row < tl.rows;
                const uint64_t po = live ? srow[row].psi : 0;
#pragma unroll
                for (int q = 0; q < kTcStageK; q++)
                    av[q] = (live && k0 + q < tl.k0) ? __ldg(psi + po + k0 + q) : 0.f;
#pragma unroll
                for (int k4 = 0; k4 < kTcStageK / 4; k4++) {
                    uint32_t h[4], l[4];
#pragma unroll
                    for (int jj = 0; jj < 4; jj++)
                        split_tf32(av[4 * k4 + jj], h[jj], l[jj]);
                    const uint32_t off = kmajor_off(row, 4 * k4);
                    *(uint4 *)(buf + off) = make_uint4(h[0], h[1], h[2], h[3]);
                    *(uint4 *)(buf + kABytes + off) = make_uint4(l[0], l[1], l[2], l[3]);
                }
            }
            // B[n][k] = op(R)(k, col0 + n)
            const uint32_t b_hi = 2 * kABytes, b_lo = b_hi + (uint32_t)tl.n * kTcStageK * 4;
            for (int nn = lane; nn < tl.n; nn += 32) {
                const int c = tl.col0 + nn;
                float bv[kTcStageK];
#pragma unroll
                for (int q = 0; q < kTcStageK; q++) {
                    const int k = k0 + q;
                    bv[q] = (c < tl.n0 && k < tl.k0)
                                ? __ldg(Rm + (tl.tb0 ? (uint64_t)c * tl.ldb0 + k : (uint64_t)k * tl.ldb0 + c))
                                : 0.f;
                }
#pragma unroll
                for (int k4 = 0; k4 < kTcStageK / 4; k4++) {
                    uint32_t h[4], l[4];
#pragma unroll
                    for (int jj = 0; jj < 4; jj++)
                        split_tf32(bv[4 * k4 + jj], h[jj], l[jj]);
                    const uint32_t off = kmajor_off(nn, 4 * k4);
                    *(uint4 *)(buf + b_hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
                    *(uint4 *)(buf + b_lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
                }
            }
            fence_async_smem();
            __syncwarp();
            if (lane == 0)
                mbar_arrive(smem_u32(&full[slot]));
        }
    } else if (warp == kMmaWarp && lane == 0) {
        const uint32_t idesc = make_idesc(tl.n);
        for (int ls = 0; ls < n_stages; ls++) {
            const int jj = ls / P, slot = ls % P + P * (jj % D), use = jj / D;
            if (!mbar_wait(smem_u32(&full[slot]), (uint32_t)(use & 1))) {
                atomicExch(err, 1);
                atomicExch(abort_flag, 1);
                break;
            }
            tc_fence_after();
            const uint32_t a_hi = smem_u32(smem + (uint32_t)slot * slot_bytes), a_lo = a_hi + kABytes;
            const uint32_t b_hi = a_hi + 2 * kABytes, b_lo = b_hi + (uint32_t)tl.n * kTcStageK * 4;
#pragma unroll
            for (int h = 0; h < kTcStageK / 8; h++) {
                const uint32_t ko = h * 2 * kLBO;
                const uint32_t acc0 = (ls > 0 || h > 0) ? 1u : 0u;
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_hi + ko), idesc, acc0);
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_lo + ko), idesc, 1u);
                mma_tf32(tmem, make_desc(a_lo + ko), make_desc(b_hi + ko), idesc, 1u);
            }
            mma_commit(smem_u32(&empty[slot]));
        }
        mma_commit(smem_u32(done));
    }
    __syncwarp();
    const int good = __syncthreads_and(mbar_wait(smem_u32(done), 0u) ? 1 : 0);
    tc_fence_after();
    if (!good && tid == 0)
        atomicExch(err, 1);
    if (good && *abort_flag == 0) {
        const int q4 = warp & 3, half = warp >> 2;
        const int trow = q4 * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(q4 * 32) << 16);
        for (int c16 = half * 16; c16 < tl.n; c16 += 32) {
            float v[16];
            tmem_ld16(tbase + (uint32_t)c16, v);
            if (trow >= tl.rows)
                continue;
            float *wrow = work + srow[trow].w + tl.col0 + c16;
            const int lim = tl.n0 - tl.col0 - c16;
#pragma unroll
            for (int j = 0; j < 16; j++)
                if (j < lim)
                    wrow[j] = v[j];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kMaxN));
}

// split-K reduction: sigma += scale * sum over chunks (fixed order); block (tile, 8-row group)
__global__ void __launch_bounds__(256) tc_reduce_kernel(const int32_t *__restrict__ multi,
                                                        const TcTile *__restrict__ tiles,
                                                        const Region *__restrict__ regions,
                                                        const float *__restrict__ part,
                                                        double *__restrict__ sigma, double scale,
                                                        RootStrides rs) {
    const TcTile tl = tiles[multi[blockIdx.x]];
    part += blockIdx.z * rs.part;
    sigma += blockIdx.z * rs.sigma;
    const Region rg = regions[tl.g];
    const int r0 = blockIdx.y * 8;
    if (r0 >= tl.rows)
        return;
    const int nr = min(8, tl.rows - r0);
    const int64_t plane = (int64_t)tl.rows * tl.n;
    for (int e = threadIdx.x; e < nr * tl.n; e += blockDim.x) {
        const int r = r0 + e / tl.n, cc = e % tl.n;
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
                             double *sigma, float *part, double scale, int *err,
                             const RootStrides &rs, cudaStream_t s) {
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
    tc_phase2_kernel<<<dim3((unsigned)p.n_tct, rs.nroots), kThreads, kSmemBytes, s>>>(
        p.tct, p.tctile, p.tcs, p.regions, ops, work, sigma, part, scale, err, rs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || p.n_tc_multi == 0)
        return e;
    tc_reduce_kernel<<<dim3((unsigned)p.n_tc_multi, 16, rs.nroots), 256, 0, s>>>(
        p.tc_multi, p.tctile, p.regions, part, sigma, scale, rs);
    return cudaGetLastError();
}

} // namespace b2g

namespace b2g {

cudaError_t launch_tc_phase1(const DevicePlan &p, const float *ops, const float *psi, float *work,
                             int *err, const RootStrides &rs, cudaStream_t s) {
    if (p.n_tc1t == 0)
        return cudaSuccess;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(tc_phase1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kSmem1Bytes);
        if (e != cudaSuccess)
            return e;
        attr_set = true;
    }
    tc_phase1_kernel<<<dim3((unsigned)p.n_tc1t, rs.nroots), kThreads, kSmem1Bytes, s>>>(
        p.tc1t, p.tc1r, ops, psi, work, err, rs);
    return cudaGetLastError();
}

} // namespace b2g
