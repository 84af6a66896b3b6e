// Tensor-core (tcgen05, kind::tf32) GEMM0 of the TF32x3 form, transposed:
// W_u^T = op(R)^T * psi_u^T for the distinct products W_u = psi_u * op(R),
// split-TF32 x3 (hi*hi + hi*lo + lo*hi) with an FP32 accumulator in TMEM.
//
// One CTA per tile (a 128-row piece of op(R)^T times up to 256 stacked psi
// rows of the products that share R), K = k0 in 16-column stages:
//   * warp 0 lane 0 bulk-copies the stage's op(R)^T slab (TF32 hi/lo,
//     canonical K-major layout, built once per H_eff) into a ring slot;
//   * warps 2..7 gather the stage's psi rows from a packed FP32 copy of the
//     psi sub-blocks (rows 16-byte aligned and zero-padded to 4 columns, made
//     per product, L2 resident) with 16-byte cp.async copies (two stages in
//     flight), then split them in shared memory into the TF32 hi/lo parts;
//   * warp 1 lane 0 waits for both (the copies' mbarrier with their byte
//     count, the gather's mbarrier), issues the six MMAs and commits them to
//     the slot's empty barrier;
//   * warps 4..7 then drain the accumulator: each thread holds one column of
//     W (a TMEM lane) and 16 stacked psi rows per tcgen05.ld, and writes every
//     4 rows as one 16-byte chunk of the W image GEMM1 reads (hi and lo).
//
// Every mbarrier wait is bounded: on timeout the kernel sets *err, waits
// (bounded) for its outstanding copies, frees its TMEM and returns.
#include "b2g_internal.h"
#include "b2g_tcgen05.cuh"

namespace b2g {

namespace {

using namespace tcg;

constexpr int kThreads = 256;
constexpr int kGatherWarp0 = 2;                      // warps 2..7 gather psi
constexpr int kGatherThreads = kThreads - 32 * kGatherWarp0;
constexpr int kMaxRing = 4;
constexpr uint32_t kABytes = 128 * kTcStageK * 4;    // one split part of the A slab (8 KB)
// two instantiations: tiles wider than 128 columns (96 KB ring, 256 TMEM
// columns, two CTAs per SM) and the rest (64 KB ring, 128 columns, three)
constexpr uint32_t kWideRing = 96 * 1024, kNarrowRing = 64 * 1024;

__device__ __forceinline__ void gather_bar() {
    asm volatile("bar.sync 1, %0;" ::"n"(kGatherThreads) : "memory");
}

// 16-byte asynchronous copy global -> shared (L2 only); src_bytes = 0 writes zeros
__device__ __forceinline__ void cp_async16(uint32_t dst, const float *src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes)
                 : "memory");
}

// psi sub-blocks -> packed FP32 copy with rows padded (zeros) to a multiple of 4
__global__ void __launch_bounds__(256) g0_pack_psi(const G0Psi *__restrict__ blocks,
                                                   const double *__restrict__ psi,
                                                   float *__restrict__ out, RootStrides rs,
                                                   uint64_t out_stride) {
    const G0Psi b = blocks[blockIdx.x];
    psi += blockIdx.y * rs.psi;
    out += blockIdx.y * out_stride;
    for (int e = threadIdx.x; e < b.m0 * b.k0p; e += blockDim.x) {
        const int i = e / b.k0p, k = e - i * b.k0p;
        out[b.dst + e] = k < b.k0 ? (float)psi[b.src + (uint64_t)i * b.lda0 + k] : 0.f;
    }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <uint32_t kRingBytes, uint32_t kTmemCols, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks)
g0_kernel(const G0Tile *__restrict__ tiles, const G0Col *__restrict__ coltab,
          const unsigned char *__restrict__ aimg, const float *__restrict__ psi,
          unsigned char *__restrict__ wimg, int *err, RootStrides rs) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ G0Col scol[256];
    __shared__ __align__(8) uint64_t full[kMaxRing], fullb[kMaxRing], empty[kMaxRing], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag, n_issued, n_consumed, gather_stop;
    psi += blockIdx.y * rs.psi;
    wimg += blockIdx.y * rs.wimg;
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const G0Tile tl = tiles[blockIdx.x];
    const int ns = tl.nsl;
    const uint32_t b_bytes = (uint32_t)tl.n * 64;
    const uint32_t slot_bytes = (2 * kABytes + 2 * b_bytes + 1023) & ~1023u;
    const int R = min(kMaxRing, (int)(kRingBytes / slot_bytes));
    const uint32_t rows8 = tl.a_bytes / 64;

    for (int i = tid; i < tl.ncol; i += kThreads)
        scol[i] = coltab[tl.cb + i];
    if (tid == 0) {
        for (int i = 0; i < R; i++) {
            mbar_init(smem_u32(&full[i]), 1);   // the copy thread's expect_tx (bytes of the A slab)
            mbar_init(smem_u32(&fullb[i]), 1);  // the gather leader (psi rows stored)
            mbar_init(smem_u32(&empty[i]), 1);
        }
        mbar_init(smem_u32(&done), 1);
        abort_flag = 0, n_issued = 0, n_consumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&tmem_slot)), "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    // A rows the copies never write (rows8 .. 127) stay zero for the whole tile
    {
        const uint32_t tail = kABytes - rows8 * 64;
        for (int sl = 0; sl < R; sl++) {
            unsigned char *a = smem + (uint32_t)sl * slot_bytes;
            for (uint32_t o = (uint32_t)tid * 16; o < tail; o += kThreads * 16) {
                *(uint4 *)(a + rows8 * 64 + o) = make_uint4(0, 0, 0, 0);
                *(uint4 *)(a + kABytes + rows8 * 64 + o) = make_uint4(0, 0, 0, 0);
            }
        }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---------------- op(R)^T slabs by bulk copy
        for (int j = 0; j < ns; j++) {
            const int slot = j % R, use = j / R;
            if (use >= 1 && !mbar_wait(smem_u32(&empty[slot]), (uint32_t)((use - 1) & 1))) {
                atomicExch(err, 1);
                atomicExch(&abort_flag, 1);
                break;
            }
            if (*(volatile int *)&abort_flag)
                break;
            const uint32_t buf = smem_u32(smem + (uint32_t)slot * slot_bytes);
            const uint32_t fb = smem_u32(&full[slot]);
            const unsigned char *src = aimg + tl.a + (uint64_t)j * rows8 * 128;
            mbar_expect_tx(fb, 2 * tl.a_bytes);
            bulk_g2s(buf, src, tl.a_bytes, fb);
            bulk_g2s(buf + kABytes, src + tl.a_bytes, tl.a_bytes, fb);
            n_issued = j + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        const uint32_t idesc = make_idesc(tl.n);
        for (int j = 0; j < ns; j++) {
            const int slot = j % R, use = j / R;
            if (!mbar_wait(smem_u32(&full[slot]), (uint32_t)(use & 1)) ||
                !mbar_wait(smem_u32(&fullb[slot]), (uint32_t)(use & 1))) {
                atomicExch(err, 1);
                atomicExch(&abort_flag, 1);
                break;
            }
            tc_fence_after();
            const uint32_t a_hi = smem_u32(smem + (uint32_t)slot * slot_bytes), a_lo = a_hi + kABytes;
            const uint32_t b_hi = a_hi + 2 * kABytes, b_lo = b_hi + b_bytes;
#pragma unroll
            for (int h = 0; h < kTcStageK / 8; h++) {
                const uint32_t ko = h * 2 * kLBO;  // K = 8 = two core matrices
                const uint32_t acc0 = (j > 0 || h > 0) ? 1u : 0u;
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_hi + ko), idesc, acc0);
                mma_tf32(tmem, make_desc(a_hi + ko), make_desc(b_lo + ko), idesc, 1u);
                mma_tf32(tmem, make_desc(a_lo + ko), make_desc(b_hi + ko), idesc, 1u);
            }
            mma_commit(smem_u32(&empty[slot]));
            n_consumed = j + 1;
        }
        mma_commit(smem_u32(&done));
    } else if (warp >= kGatherWarp0) {
        // ---------------- psi rows (B, N x 16 per stage): 4-byte cp.async copies
        // straight into the slot's hi region (zero-filled where a row or K
        // column is padding), two stages in flight; the stage before is then
        // split in place (hi) and into the lo region, and released to the MMA
        const int gt = tid - 32 * kGatherWarp0;
        const int ne = tl.n * kTcStageK / 4;
        bool stop = false;
        for (int j = 0; j <= ns && !stop; j++) {
            if (j < ns) {
                const int slot = j % R, use = j / R;
                if (use >= 1) {
                    // the leader's decision reaches every gather thread through
                    // gather_stop, so they leave the loop together
                    if (gt == 0) {
                        if (!mbar_wait(smem_u32(&empty[slot]), (uint32_t)((use - 1) & 1))) {
                            atomicExch(err, 1);
                            atomicExch(&abort_flag, 1);
                        }
                        gather_stop = *(volatile int *)&abort_flag;
                    }
                    gather_bar();
                    stop = gather_stop != 0;
                }
                if (!stop) {
                    const uint32_t buf = smem_u32(smem + (uint32_t)slot * slot_bytes + 2 * kABytes);
                    const int k0 = j * kTcStageK;
                    for (int e = gt; e < ne; e += kGatherThreads) {
                        // one 16-byte chunk (4 K columns of one row) of the packed psi
                        // copy, whose rows are zero-padded to a multiple of 4 columns
                        const int c = e >> 2, kq = 4 * (e & 3), k = k0 + kq;
                        const bool ok = c < tl.ncol && k < tl.k0 && scol[c].live;
                        cp_async16(buf + kmajor_off(c, kq), ok ? psi + scol[c].psi + k : psi, ok ? 16u : 0u);
                    }
                }
                cp_async_commit();
            }
            if (j >= 1 && !stop) {
                if (j < ns)
                    cp_async_wait1();
                else
                    cp_async_wait0();
                gather_bar();
                const int slot = (j - 1) % R;
                unsigned char *buf = smem + (uint32_t)slot * slot_bytes + 2 * kABytes;
                for (int q = gt; q < tl.n * 4; q += kGatherThreads) {
                    const float4 x = *(const float4 *)(buf + q * 16);
                    uint32_t h[4], l[4];
                    split_tf32(x.x, h[0], l[0]);
                    split_tf32(x.y, h[1], l[1]);
                    split_tf32(x.z, h[2], l[2]);
                    split_tf32(x.w, h[3], l[3]);
                    *(uint4 *)(buf + q * 16) = make_uint4(h[0], h[1], h[2], h[3]);
                    *(uint4 *)(buf + b_bytes + q * 16) = make_uint4(l[0], l[1], l[2], l[3]);
                }
                fence_async_smem();
                gather_bar();
                if (gt == 0)
                    mbar_arrive(smem_u32(&fullb[slot]));
            }
        }
        cp_async_wait0();  // nothing may land after the CTA has moved on
    }
    // ---- epilogue: warps 4..7 own TMEM lane quarters (warp & 3)
    __syncwarp();
    const int good = __syncthreads_and(mbar_wait(smem_u32(&done), 0u) ? 1 : 0);
    tc_fence_after();
    if (!good && tid == 0)
        atomicExch(err, 1);
    if (good && abort_flag == 0 && warp >= 4) {
        const int q4 = warp & 3;
        const int m = q4 * 32 + lane;               // W column m_off + m
        const uint32_t tbase = tmem + ((uint32_t)(q4 * 32) << 16);
        const int nw = tl.m_off + m;
        for (int c16 = 0; c16 < tl.n; c16 += 16) {
            float v[16];
            tmem_ld16(tbase + (uint32_t)c16, v);
            if (m >= tl.rows)
                continue;
#pragma unroll
            for (int g = 0; g < 4; g++) {
                const int c = c16 + 4 * g;
                if (c >= tl.ncol)
                    break;
                const G0Col cl = scol[c];           // first of 4 rows of one product (k % 4 == 0)
                unsigned char *base = wimg + cl.w + (uint64_t)(cl.k >> 4) * tl.npad * 128 +
                                      kmajor_off(nw, cl.k & 15);
                uint32_t h[4], l[4];
#pragma unroll
                for (int i = 0; i < 4; i++)
                    split_tf32(v[4 * g + i], h[i], l[i]);
                *(uint4 *)base = make_uint4(h[0], h[1], h[2], h[3]);
                *(uint4 *)(base + tl.npad * 64) = make_uint4(l[0], l[1], l[2], l[3]);
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
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

} // namespace

template <uint32_t kRingBytes, uint32_t kTmemCols, int kMinBlocks>
static cudaError_t launch_g0_class(const G0Tile *tiles, int64_t n, const DevicePlan &p,
                                   const unsigned char *aimg, const float *psi_packed,
                                   unsigned char *wimg, int *err, const RootStrides &rs, cudaStream_t s) {
    if (n == 0)
        return cudaSuccess;
    constexpr uint32_t smem = kRingBytes + 1024;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(g0_kernel<kRingBytes, kTmemCols, kMinBlocks>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
        attr_set = true;
    }
    note_launch();
    g0_kernel<kRingBytes, kTmemCols, kMinBlocks><<<dim3((unsigned)n, rs.nroots), kThreads, smem, s>>>(
        tiles, p.g0col, aimg, psi_packed, wimg, err, rs);
    return cudaGetLastError();
}

cudaError_t launch_g0(const DevicePlan &p, const unsigned char *aimg, const double *psi,
                      float *psi_packed, unsigned char *wimg, int *err, const RootStrides &rs,
                      cudaStream_t s) {
    if (p.n_g0tile == 0)
        return cudaSuccess;
    note_launch();
    g0_pack_psi<<<dim3((unsigned)p.n_g0psi, rs.nroots), 256, 0, s>>>(p.g0psi, psi, psi_packed, rs,
                                                                    p.g0_psi_floats);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    RootStrides rp = rs;
    rp.psi = p.g0_psi_floats;  // the kernels read the packed copy
    // tiles [0, n_g0wide) are wider than 128 columns, the rest are not
    if ((e = launch_g0_class<kWideRing, 256, 2>(p.g0tile, p.n_g0wide, p, aimg, psi_packed, wimg, err,
                                                rp, s)) != cudaSuccess)
        return e;
    return launch_g0_class<kNarrowRing, 128, 3>(p.g0tile + p.n_g0wide, p.n_g0tile - p.n_g0wide, p, aimg,
                                                psi_packed, wimg, err, rp, s);
}

} // namespace b2g
