// Tensor-core (tcgen05, kind::tf32) GEMM0 of the TF32x3 form:
// W_u = psi_sub * op(R) for the distinct products, split-TF32 x3 (hi*hi +
// hi*lo + lo*hi) with FP32 accumulation in TMEM.
//
// One CTA per tile: up to 128 rows of products that share one right
// operator block R, stacked along M, times <= 256 columns of R.  Producer
// warps gather the psi rows and the R slab of each 16-column K stage from
// the FP32 copies, split them into TF32 hi/lo parts and write them into a
// ring of shared-memory stage slots in the canonical no-swizzle K-major
// layout; lane 0 of the MMA warp waits for a slot (mbarrier), issues the
// stage's six MMAs and commits them to the slot's empty barrier; all warps
// drain the accumulator (tcgen05.ld) into the FP32 work rows.
//
// Every mbarrier wait is bounded: on timeout the kernel sets *err, waits
// (bounded) for its outstanding MMAs, frees its TMEM and returns.
#include "b2g_internal.h"
#include "b2g_tcgen05.cuh"

namespace b2g {

namespace {

using namespace tcg;

constexpr int kThreads = 256;                          // 8 warps
constexpr int kProducers = 7;                          // warps 0..6 stage operands
constexpr int kMmaWarp = 7;                            // lane 0 of warp 7 issues the MMAs
constexpr int kMaxN = 256;
constexpr int kMaxRing = 8;
constexpr uint32_t kABytes = 128 * kTcStageK * 4;      // 8 KB per split part of A
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

} // namespace

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
