// Image-fed tensor-core GEMM1 of the TF32x3 form: sigma += scale * sum over
// pairs of alpha * op(L) * W_u, on tcgen05 (kind::tf32, three products per
// split operand pair, FP32 accumulator in TMEM).
//
// The operands are prepared in HBM as exactly the shared-memory tiles the MMA
// reads (TF32 hi/lo split, canonical no-swizzle K-major core-matrix layout),
// so a stage is four contiguous bulk copies (cp.async.bulk, completing on an
// mbarrier) issued by one thread: no per-element loads, conversions or
// predicates in the main loop.
//   * A images: alpha * op(L) for each distinct (operator block, alpha),
//     built once per H_eff from the FP32 operator copy (g1_build_a).
//   * W images: W_u^T per 16-row K slab, written per product by the GEMM0
//     kernel's epilogue (b2g_tc.cu).
// One CTA per chunk (at most kG1ChunkStages slabs of one tile): warp 0 lane 0
// issues the copies into a ring of stage slots, warp 1 lane 0 waits for a
// slot, issues its six MMAs and commits them to the slot's empty barrier,
// warps 2..5 drain the accumulator into the chunk's partial tile.  A
// reduction kernel then adds, per sigma cell, the partials of every tile
// covering it in a fixed order (deterministic).
//
// Every mbarrier wait is bounded; on timeout the kernel sets *err, waits
// (bounded) for the copies it issued, frees its TMEM and returns.
#include "b2g_internal.h"
#include "b2g_tcgen05.cuh"

namespace b2g {

namespace {

using namespace tcg;

constexpr int kG1Threads = 192;                 // warp 0 copies, warp 1 MMAs, warps 2..5 epilogue
constexpr int kG1MaxRing = 6;
constexpr uint32_t kG1ABytes = 128 * kG1SlabK * 4;   // one split part of the A slab (8 KB)
constexpr uint32_t kG1RingBytes = 96 * 1024;         // two CTAs per SM
constexpr int kG1MaxStages = kG1ChunkLimit;          // stage table held in shared memory
constexpr uint32_t kG1SmemBytes = kG1RingBytes + 1024;
constexpr uint32_t kG1TmemCols = 256;

__global__ void __launch_bounds__(256) g1_build_a(const G1AImg *__restrict__ imgs,
                                                  const float *__restrict__ ops,
                                                  unsigned char *__restrict__ out) {
    const G1AImg im = imgs[blockIdx.x];
    const int ns = (im.k1 + kG1SlabK - 1) / kG1SlabK;
    const int npieces = (im.m1 + 127) / 128;
    const float *L = ops + im.src;
    for (int rp = 0; rp < npieces; rp++) {
        const int rows = min(128, im.m1 - 128 * rp), rows8 = (rows + 7) & ~7;
        for (int sl = 0; sl < ns; sl++) {
            unsigned char *base = out + im.dst + (uint64_t)rp * 16384 * ns + (uint64_t)sl * rows8 * 128;
            for (int e = threadIdx.x; e < rows8 * kG1SlabK; e += blockDim.x) {
                const int m = e >> 4, k = e & 15;
                const int mg = 128 * rp + m, kg = kG1SlabK * sl + k;
                float v = 0.f;
                if (m < rows && kg < im.k1)
                    v = im.alpha * L[im.ta1 ? (uint64_t)kg * im.lda1 + mg : (uint64_t)mg * im.lda1 + kg];
                uint32_t hi, lo;
                split_tf32(v, hi, lo);
                const uint32_t off = kmajor_off(m, k);
                *(uint32_t *)(base + off) = hi;
                *(uint32_t *)(base + rows8 * 64 + off) = lo;
            }
        }
    }
}

__global__ void __launch_bounds__(kG1Threads, 2)
g1_kernel(const G1Task *__restrict__ tasks, const G1Tile *__restrict__ tiles,
          const G1Stage *__restrict__ stages, const unsigned char *__restrict__ aimg,
          const unsigned char *__restrict__ wimg, float *__restrict__ part, int *err,
          RootStrides rs) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ G1Stage sst[kG1MaxStages];
    __shared__ __align__(8) uint64_t full[kG1MaxRing], empty[kG1MaxRing], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag, n_issued, n_consumed;
    wimg += blockIdx.y * rs.wimg;
    part += blockIdx.y * rs.part;
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const G1Task tk = tasks[blockIdx.x];
    const G1Tile tl = tiles[tk.tile];
    const int ns = tk.n_stages;
    const uint32_t b_bytes = (uint32_t)tl.n * 64;
    const uint32_t slot_bytes = (2 * kG1ABytes + 2 * b_bytes + 1023) & ~1023u;
    const int R = min(kG1MaxRing, (int)(kG1RingBytes / slot_bytes));
    const uint32_t rows8 = (uint32_t)((tl.rows + 7) & ~7);

    for (int i = tid; i < ns; i += kG1Threads)
        sst[i] = stages[tk.st0 + i];
    if (tid == 0) {
        for (int i = 0; i < R; i++) {
            mbar_init(smem_u32(&full[i]), 1);
            mbar_init(smem_u32(&empty[i]), 1);
        }
        mbar_init(smem_u32(&done), 1);
        abort_flag = 0, n_issued = 0, n_consumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&tmem_slot)), "r"(kG1TmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // rows the copies never write (rows8 .. 127 of A) stay zero for the whole tile
    {
        const uint32_t tail = kG1ABytes - rows8 * 64;
        for (int sl = 0; sl < R; sl++) {
            unsigned char *a = smem + (uint32_t)sl * slot_bytes;
            for (uint32_t o = (uint32_t)tid * 16; o < tail; o += kG1Threads * 16) {
                *(uint4 *)(a + rows8 * 64 + o) = make_uint4(0, 0, 0, 0);
                *(uint4 *)(a + kG1ABytes + rows8 * 64 + o) = make_uint4(0, 0, 0, 0);
            }
        }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------- bulk-copy producer
        for (int j = 0; j < ns; j++) {
            const int slot = j % R, use = j / R;
            if (use >= 1 && !mbar_wait(smem_u32(&empty[slot]), (uint32_t)((use - 1) & 1))) {
                atomicExch(err, 1);
                atomicExch(&abort_flag, 1);
                break;
            }
            if (*(volatile int *)&abort_flag)
                break;
            const G1Stage st = sst[j];
            const uint32_t buf = smem_u32(smem + (uint32_t)slot * slot_bytes);
            const uint32_t fb = smem_u32(&full[slot]);
            mbar_expect_tx(fb, 2 * st.a_bytes + 2 * b_bytes);
            bulk_g2s(buf, aimg + st.a, st.a_bytes, fb);
            bulk_g2s(buf + kG1ABytes, aimg + st.a + st.a_bytes, st.a_bytes, fb);
            bulk_g2s(buf + 2 * kG1ABytes, wimg + st.b, b_bytes, fb);
            bulk_g2s(buf + 2 * kG1ABytes + b_bytes, wimg + st.b + st.b_lo, b_bytes, fb);
            n_issued = j + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        const uint32_t idesc = make_idesc(tl.n);
        for (int j = 0; j < ns; j++) {
            const int slot = j % R, use = j / R;
            if (!mbar_wait(smem_u32(&full[slot]), (uint32_t)(use & 1))) {
                atomicExch(err, 1);
                atomicExch(&abort_flag, 1);
                break;
            }
            tc_fence_after();
            const uint32_t a_hi = smem_u32(smem + (uint32_t)slot * slot_bytes), a_lo = a_hi + kG1ABytes;
            const uint32_t b_hi = a_hi + 2 * kG1ABytes, b_lo = b_hi + b_bytes;
#pragma unroll
            for (int h = 0; h < kG1SlabK / 8; h++) {
                const uint32_t ko = h * 2 * kLBO;  // K = 8 = two core matrices
                const uint32_t acc0 = (j > 0 || h > 0) ? 1u : 0u;
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_hi + ko), idesc, acc0);
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_lo + ko), idesc, 1u);
                mma_tf32(tmem, make_desc(a_lo + ko), make_desc(b_hi + ko), idesc, 1u);
            }
            mma_commit(smem_u32(&empty[slot]));
            n_consumed = j + 1;
        }
        mma_commit(smem_u32(&done));  // tracks every MMA issued above
    }
    // ---- epilogue: warps 2..5 own TMEM lane quarters (warp & 3)
    __syncwarp();
    const int good = __syncthreads_and(mbar_wait(smem_u32(&done), 0u) ? 1 : 0);
    tc_fence_after();
    if (!good && tid == 0)
        atomicExch(err, 1);
    if (good && abort_flag == 0 && warp >= 2) {
        const int q4 = warp & 3;
        const int trow = q4 * 32 + lane;
        const uint32_t tbase = tmem + ((uint32_t)(q4 * 32) << 16);
        float *prow = part + tl.part + ((int64_t)tk.chunk * tl.rows + trow) * tl.n;
        for (int c16 = 0; c16 < tl.n; c16 += 16) {
            float v[16];
            tmem_ld16(tbase + (uint32_t)c16, v);
            if (trow < tl.rows) {
#pragma unroll
                for (int j = 0; j < 16; j += 4)
                    *(float4 *)(prow + c16 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (abort_flag && tid == 0) {
        // copies issued but never consumed must land before the CTA exits
        for (int j = n_consumed; j < n_issued; j++)
            mbar_wait(smem_u32(&full[j % R]), (uint32_t)((j / R) & 1));
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kG1TmemCols));
}

// sigma += scale * (sum of the partials of every tile covering the cell), per
// reduction item (rows [r0, r1) of one region, with the list of the tiles that
// meet those rows), tiles and chunks in fixed order.  The partials are summed
// in FP32 with Kahan compensation (FP64 adds would run on GB300's narrow FP64
// pipe) and added to sigma in FP64.
constexpr int kRedTiles = 64;
__global__ void __launch_bounds__(256) g1_reduce(const G1Red *__restrict__ items,
                                                 const int32_t *__restrict__ cover,
                                                 const G1Tile *__restrict__ tiles,
                                                 const Region *__restrict__ regions,
                                                 const float *__restrict__ part,
                                                 double *__restrict__ sigma, double scale,
                                                 RootStrides rs) {
    __shared__ G1Tile st[kRedTiles];
    const G1Red it = items[blockIdx.x];
    part += blockIdx.y * rs.part;
    sigma += blockIdx.y * rs.sigma;
    const Region rg = regions[it.g];
    const int nt = it.t1 - it.t0;
    for (int i = threadIdx.x; i < min(nt, kRedTiles); i += blockDim.x)
        st[i] = tiles[cover[it.t0 + i]];
    __syncthreads();
    const int nr = it.r1 - it.r0;
    for (int e = threadIdx.x; e < nr * rg.cols; e += blockDim.x) {
        const int r = it.r0 + e / rg.cols, c = e % rg.cols;
        const uint64_t a = rg.base + (uint64_t)r * rg.ld + (uint64_t)c;
        if (a < rg.lo || a >= rg.hi)
            continue;
        float s = 0.f, comp = 0.f;
        bool covered = false;
        for (int q = 0; q < nt; q++) {
            const G1Tile tl = q < kRedTiles ? st[q] : tiles[cover[it.t0 + q]];
            const int rr = r - tl.row0, cc = c - tl.col0;
            if (rr < 0 || rr >= tl.rows || cc < 0 || cc >= tl.ncols)
                continue;
            covered = true;
            const float *p = part + tl.part + (int64_t)rr * tl.n + cc;
            const int64_t plane = (int64_t)tl.rows * tl.n;
            // eight chunk loads in flight, then their compensated adds in order
            for (int ch0 = 0; ch0 < tl.n_chunks; ch0 += 8) {
                float x[8];
#pragma unroll
                for (int i = 0; i < 8; i++)
                    x[i] = ch0 + i < tl.n_chunks ? __ldg(p + (ch0 + i) * plane) : 0.f;
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const float y = x[i] - comp;
                    const float t = s + y;
                    comp = (t - s) - y;
                    s = t;
                }
            }
        }
        if (covered)
            sigma[a] += scale * ((double)s - (double)comp);
    }
}

} // namespace

cudaError_t launch_g1_build_a(const DevicePlan &p, const float *ops32, unsigned char *aimg,
                              cudaStream_t s) {
    if (p.n_g1aimg == 0)
        return cudaSuccess;
    note_launch();
    g1_build_a<<<(unsigned)p.n_g1aimg, 256, 0, s>>>(p.g1aimg, ops32, aimg);
    return cudaGetLastError();
}

cudaError_t launch_g1(const DevicePlan &p, const unsigned char *aimg, const unsigned char *wimg,
                      float *part, double *sigma, double scale, int *err, const RootStrides &rs,
                      cudaStream_t s) {
    if (p.n_g1task == 0)
        return cudaSuccess;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(g1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kG1SmemBytes);
        if (e != cudaSuccess)
            return e;
        attr_set = true;
    }
    note_launch();
    g1_kernel<<<dim3((unsigned)p.n_g1task, rs.nroots), kG1Threads, kG1SmemBytes, s>>>(
        p.g1task, p.g1tile, p.g1stage, aimg, wimg, part, err, rs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    note_launch();
    g1_reduce<<<dim3((unsigned)p.n_g1red, rs.nroots), 256, 0, s>>>(p.g1red, p.g1cover, p.g1tile,
                                                                  p.regions, part, sigma, scale, rs);
    return cudaGetLastError();
}

} // namespace b2g
