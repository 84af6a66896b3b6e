// CUDA-core forms of H_eff*psi on sm_103a: plain FP64 (DFMA) and FP32 (FFMA).
//
// GB300 executes FP64 on CUDA-core DFMA units only (no FP64 tensor path), at
// a small fraction of its tensor rate, so the FP64 kernels are DFMA-issue
// bound: the design goal is that every issued DFMA lane does useful work (no
// padded tiles) and that enough independent warps are resident to hide
// latency.  Operands are re-read through L1/L2 (the operator blocks of one
// H_eff are reused by many pairs and stay L2-resident).
//
// The FP32 instantiation (operators pre-rounded to float once per plan, W in
// float, FP32 accumulation, sigma updated in FP64) is the CUDA-core
// counterpart of the tensor-core mixed form and shares its error model.
#include "b2g_internal.h"

namespace b2g {

namespace {

constexpr int kLanesCols = 8;  // column chunks of 32 per warp (256 columns)

// Phase 1: one warp per row r of a distinct product W_u (m0 x n0):
//   W_u[r, c] = sum_k psi[a0 + r*lda0 + k] * B(k, c),
//   B(k, c) = ops[b0 + k*ldb0 + c] (tb0 = 0) or ops[b0 + c*ldb0 + k] (tb0 = 1).
// psi loads are warp-broadcast; B loads are coalesced for tb0 = 0 and
// L1-served column walks for tb0 = 1.  A predicated-off FMA still occupies
// the FP64 pipe for a whole warp instruction, so the number of column chunks
// (NJ) is a compile-time, warp-uniform count: every issued FMA carries at
// least one live column.
template <typename T, int NJ>
__device__ __forceinline__ void p1_chunk(const T *__restrict__ prow, const T *__restrict__ B,
                                         const WorkDesc &wd, int cbase, int lane,
                                         T *__restrict__ wrow) {
    T acc[NJ];
    int col[NJ];
    bool live[NJ];
#pragma unroll
    for (int j = 0; j < NJ; j++) {
        acc[j] = T(0);
        col[j] = cbase + lane + 32 * j;
        live[j] = col[j] < wd.n0;
    }
    if (!wd.tb0) {
        for (int k = 0; k < wd.k0; k++) {
            const T a = __ldg(prow + k);
            const T *brow = B + (uint64_t)k * wd.ldb0 + cbase + lane;
#pragma unroll
            for (int j = 0; j < NJ; j++)
                if (live[j])
                    acc[j] = fma(a, __ldg(brow + 32 * j), acc[j]);
        }
    } else {
        for (int k = 0; k < wd.k0; k++) {
            const T a = __ldg(prow + k);
#pragma unroll
            for (int j = 0; j < NJ; j++)
                if (live[j])
                    acc[j] = fma(a, __ldg(B + (uint64_t)col[j] * wd.ldb0 + k), acc[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < NJ; j++)
        if (live[j])
            wrow[col[j]] = acc[j];
}

template <typename T>
__global__ void __launch_bounds__(128) simt_phase1(const WorkDesc *__restrict__ works,
                                                   const Task1 *__restrict__ tasks, int64_t n_tasks,
                                                   const T *__restrict__ ops,
                                                   const T *__restrict__ psi,
                                                   T *__restrict__ work, RootStrides rs) {
    const int64_t t = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (t >= n_tasks)
        return;
    psi += blockIdx.y * rs.psi;
    work += blockIdx.y * rs.work;
    const Task1 tk = tasks[t];
    const WorkDesc wd = works[tk.u];
    const T *prow = psi + wd.a0 + (uint64_t)tk.r * wd.lda0;
    const T *B = ops + wd.b0;
    T *wrow = work + wd.woff + (uint64_t)tk.r * wd.n0;
    for (int cbase = 0; cbase < wd.n0; cbase += 32 * kLanesCols) {
        switch (min(kLanesCols, (wd.n0 - cbase + 31) >> 5)) {
        case 1: p1_chunk<T, 1>(prow, B, wd, cbase, lane, wrow); break;
        case 2: p1_chunk<T, 2>(prow, B, wd, cbase, lane, wrow); break;
        case 3: p1_chunk<T, 3>(prow, B, wd, cbase, lane, wrow); break;
        case 4: p1_chunk<T, 4>(prow, B, wd, cbase, lane, wrow); break;
        case 5: p1_chunk<T, 5>(prow, B, wd, cbase, lane, wrow); break;
        case 6: p1_chunk<T, 6>(prow, B, wd, cbase, lane, wrow); break;
        case 7: p1_chunk<T, 7>(prow, B, wd, cbase, lane, wrow); break;
        default: p1_chunk<T, 8>(prow, B, wd, cbase, lane, wrow); break;
        }
    }
}

// Phase 2: one CTA per task (4 rows x 256 columns of one sigma region, one
// chunk of its contribution list), one warp per row, lane -> columns
// lane + 32 j.  The task loops over its chunk (pairs whose row window covers
// its rows) and adds alpha * sum_k A(r - row0, k) * W_u(k, c - col0) in a
// fixed order.  A tile with a single chunk owns its cells and writes
// sigma += scale * acc directly; otherwise the chunk stores its partial tile
// and simt_reduce sums the chunks in order.  Only cells inside the region's
// write span are stored (no atomics, deterministic).
//
// Per contribution only the column chunks [J0, J1) that meet its columns are
// issued (compile-time range picked by a warp-uniform dispatch), the dot
// products are summed unscaled and alpha is applied once per contribution,
// so the FP64 pipe issues no FMA without a live column and no per-k multiply.
template <typename T, int J0, int J1>
__device__ __forceinline__ void p2_contrib(T (&acc)[kLanesCols], const T *__restrict__ A,
                                           const T *__restrict__ W, const Contrib &c, int ar,
                                           int colbase) {
    constexpr int NJ = J1 - J0;
    T t[NJ];
    int col[NJ];
    bool live[NJ];
#pragma unroll
    for (int j = 0; j < NJ; j++) {
        t[j] = T(0);
        col[j] = colbase + 32 * (J0 + j);
        live[j] = col[j] >= 0 && col[j] < c.n1;
    }
    const uint64_t astep = c.ta1 ? (uint64_t)c.lda1 : 1;
    const T *ap = A + (c.ta1 ? (uint64_t)ar : (uint64_t)ar * c.lda1);
    for (int k = 0; k < c.k1; k++) {
        const T a = __ldg(ap + (uint64_t)k * astep);
        const T *wrow = W + (uint64_t)k * c.n1;
#pragma unroll
        for (int j = 0; j < NJ; j++)
            if (live[j])
                t[j] = fma(a, __ldg(wrow + col[j]), t[j]);
    }
    const T alpha = (T)c.alpha;
#pragma unroll
    for (int j = 0; j < NJ; j++)
        acc[J0 + j] = fma(alpha, t[j], acc[J0 + j]);
}

template <typename T, int J0, int J1>
__device__ __forceinline__ void p2_pick_j1(int j1, T (&acc)[kLanesCols], const T *A, const T *W,
                                           const Contrib &c, int ar, int colbase) {
    if constexpr (J1 <= kLanesCols) {
        if (j1 == J1)
            p2_contrib<T, J0, J1>(acc, A, W, c, ar, colbase);
        else
            p2_pick_j1<T, J0, J1 + 1>(j1, acc, A, W, c, ar, colbase);
    }
}

template <typename T, int J0>
__device__ __forceinline__ void p2_pick(int j0, int j1, T (&acc)[kLanesCols], const T *A,
                                        const T *W, const Contrib &c, int ar, int colbase) {
    if constexpr (J0 < kLanesCols) {
        if (j0 == J0)
            p2_pick_j1<T, J0, J0 + 1>(j1, acc, A, W, c, ar, colbase);
        else
            p2_pick<T, J0 + 1>(j0, j1, acc, A, W, c, ar, colbase);
    }
}

template <typename T>
__global__ void __launch_bounds__(128) simt_phase2(const Task2 *__restrict__ tasks,
                                                   const int32_t *__restrict__ lists,
                                                   const Contrib *__restrict__ contribs,
                                                   const Region *__restrict__ regions,
                                                   const WorkDesc *__restrict__ works,
                                                   const T *__restrict__ ops,
                                                   const T *__restrict__ work,
                                                   double *__restrict__ sigma, T *__restrict__ part,
                                                   double scale, RootStrides rs) {
    const Task2 tk = tasks[blockIdx.x];
    work += blockIdx.y * rs.work;
    sigma += blockIdx.y * rs.sigma;
    part += blockIdx.y * rs.part;
    const Region rg = regions[tk.g];
    const int lane = threadIdx.x & 31;
    const int wr = threadIdx.x >> 5;
    const int r = tk.rb * 4 + wr;
    if (r >= rg.rows)
        return;
    T acc[kLanesCols];
#pragma unroll
    for (int j = 0; j < kLanesCols; j++)
        acc[j] = T(0);
    for (int64_t li = tk.lb; li < tk.le; li++) {
        const Contrib c = contribs[lists[li]];
        const int ar = r - c.row0;
        if (ar < 0 || ar >= c.m1)
            continue;  // warp-uniform
        // column chunks of the window [tk.col0, tk.col0 + 256) meeting the
        // contribution's columns [c.col0, c.col0 + n1)
        const int lo = c.col0 - tk.col0, hi = lo + c.n1;
        const int j0 = lo > 0 ? lo >> 5 : 0;
        const int j1 = min(kLanesCols, (hi + 31) >> 5);
        if (j1 <= j0)
            continue;
        p2_pick<T, 0>(j0, j1, acc, ops + c.a1, work + works[c.u].woff, c, ar, tk.col0 + lane - c.col0);
    }
    if (tk.part >= 0) {
        T *prow = part + ((tk.part + tk.chunk) * 4 + wr) * (int64_t)(32 * kLanesCols);
#pragma unroll
        for (int j = 0; j < kLanesCols; j++)
            prow[lane + 32 * j] = acc[j];
        return;
    }
    const uint64_t rowaddr = rg.base + (uint64_t)r * rg.ld;
#pragma unroll
    for (int j = 0; j < kLanesCols; j++) {
        const int col = tk.col0 + lane + 32 * j;
        const uint64_t a = rowaddr + (uint64_t)col;
        if (col < rg.cols && a >= rg.lo && a < rg.hi)
            sigma[a] += scale * (double)acc[j];
    }
}

// split-K reduction of phase 2: sigma += scale * sum over chunks (in order)
template <typename T>
__global__ void __launch_bounds__(128) simt_reduce(const Tile2 *__restrict__ tiles,
                                                   const Region *__restrict__ regions,
                                                   const T *__restrict__ part,
                                                   double *__restrict__ sigma, double scale,
                                                   RootStrides rs) {
    const Tile2 tl = tiles[blockIdx.x];
    part += blockIdx.y * rs.part;
    sigma += blockIdx.y * rs.sigma;
    const Region rg = regions[tl.g];
    const int lane = threadIdx.x & 31, wr = threadIdx.x >> 5;
    const int r = tl.rb * 4 + wr;
    if (r >= rg.rows)
        return;
    const uint64_t rowaddr = rg.base + (uint64_t)r * rg.ld;
    for (int j = 0; j < kLanesCols; j++) {
        const int col = tl.col0 + lane + 32 * j;
        const uint64_t a = rowaddr + (uint64_t)col;
        if (col >= rg.cols || a < rg.lo || a >= rg.hi)
            continue;
        double s = 0.0;
        for (int ch = 0; ch < tl.n_chunks; ch++)
            s += (double)part[((tl.part + ch) * 4 + wr) * (int64_t)(32 * kLanesCols) + lane + 32 * j];
        sigma[a] += scale * s;
    }
}

// FP64 ceiling probe: 8 independent FMA chains per thread, no memory traffic
__global__ void __launch_bounds__(256) fp64_fma_loop(double *out, int iters, double x, double y) {
    double a[8];
#pragma unroll
    for (int j = 0; j < 8; j++)
        a[j] = threadIdx.x * 1e-3 + j;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int j = 0; j < 8; j++)
            a[j] = fma(a[j], x, y);
    double s = 0;
#pragma unroll
    for (int j = 0; j < 8; j++)
        s += a[j];
    if (s == 12345.678)  // never true: keeps the loop live
        out[0] = s;
}

// FP64 tensor-core (DMMA) throughput: eight independent accumulator chains of
// mma.sync m8n8k4 f64 per warp (512 FLOP per warp instruction), registers only.
__global__ void __launch_bounds__(256) fp64_mma_loop(double *out, int iters) {
    const double a = 1.0 + threadIdx.x * 1e-9, b = 0.999999;
    double c[8][2];
#pragma unroll
    for (int j = 0; j < 8; j++)
        c[j][0] = j * 1e-3, c[j][1] = -j * 1e-3;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int j = 0; j < 8; j++)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(c[j][0]), "+d"(c[j][1])
                         : "d"(a), "d"(b));
    double s = 0;
#pragma unroll
    for (int j = 0; j < 8; j++)
        s += c[j][0] + c[j][1];
    if (s == 12345.678)  // never true: keeps the loop live
        out[0] = s;
}

__global__ void to_float(const double *__restrict__ x, float *__restrict__ y, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        y[i] = (float)x[i];
}

} // namespace

cudaError_t probe_fp64_peak(cudaStream_t s, int n_sm, double *tflops) {
    double *out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(double));
    if (e != cudaSuccess)
        return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a), cudaEventCreate(&b);
    const int blocks = n_sm * 8, iters = 4096;
    note_launch();
    fp64_fma_loop<<<blocks, 256, 0, s>>>(out, iters, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(a, s);
    note_launch();
    fp64_fma_loop<<<blocks, 256, 0, s>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(b, s);
    e = cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    *tflops = 2.0 * 8.0 * iters * (double)blocks * 256 / (ms * 1e-3) / 1e12;
    cudaEventDestroy(a), cudaEventDestroy(b);
    cudaFree(out);
    if (e == cudaSuccess)
        e = cudaGetLastError();
    return e;
}

cudaError_t probe_fp64_mma_peak(cudaStream_t s, int n_sm, double *tflops) {
    double *out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(double));
    if (e != cudaSuccess)
        return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a), cudaEventCreate(&b);
    const int blocks = n_sm * 8, iters = 1024;
    note_launch();
    fp64_mma_loop<<<blocks, 256, 0, s>>>(out, iters);  // warm-up
    cudaEventRecord(a, s);
    note_launch();
    fp64_mma_loop<<<blocks, 256, 0, s>>>(out, iters);
    cudaEventRecord(b, s);
    e = cudaEventSynchronize(b);
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    // per warp instruction 8 x 8 x 4 multiply-adds; 8 per iteration; 8 warps per block
    *tflops = 2.0 * 256.0 * 8.0 * iters * (double)blocks * 8 / (ms * 1e-3) / 1e12;
    cudaEventDestroy(a), cudaEventDestroy(b);
    cudaFree(out);
    if (e == cudaSuccess)
        e = cudaGetLastError();
    return e;
}

cudaError_t launch_to_float(const double *x, float *y, uint64_t n, cudaStream_t s) {
    if (n == 0)
        return cudaSuccess;
    const uint64_t b = (n + 255) / 256;
    note_launch();
    to_float<<<(unsigned)(b < 152 * 16 ? b : 152 * 16), 256, 0, s>>>(x, y, n);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_simt_phase1(const DevicePlan &p, const T *ops, const T *psi, T *work,
                               const RootStrides &rs, cudaStream_t s) {
    if (p.n_t1 == 0)
        return cudaSuccess;
    const int64_t blocks = (p.n_t1 + 3) / 4;
    note_launch();
    simt_phase1<T><<<dim3((unsigned)blocks, rs.nroots), 128, 0, s>>>(p.works, p.t1, p.n_t1, ops, psi,
                                                                     work, rs);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_simt_phase2(const DevicePlan &p, const T *ops, const T *work, double *sigma,
                               T *part, double scale, const RootStrides &rs, cudaStream_t s) {
    if (p.n_t2 == 0)
        return cudaSuccess;
    note_launch();
    simt_phase2<T><<<dim3((unsigned)p.n_t2, rs.nroots), 128, 0, s>>>(
        p.t2, p.lists, p.contribs, p.regions, p.works, ops, work, sigma, part, scale, rs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || p.n_t2multi == 0)
        return e;
    note_launch();
    simt_reduce<T><<<dim3((unsigned)p.n_t2multi, rs.nroots), 128, 0, s>>>(p.t2multi, p.regions, part,
                                                                          sigma, scale, rs);
    return cudaGetLastError();
}

template cudaError_t launch_simt_phase1<double>(const DevicePlan &, const double *, const double *,
                                                double *, const RootStrides &, cudaStream_t);
template cudaError_t launch_simt_phase1<float>(const DevicePlan &, const float *, const float *,
                                               float *, const RootStrides &, cudaStream_t);
template cudaError_t launch_simt_phase2<double>(const DevicePlan &, const double *, const double *,
                                                double *, double *, double, const RootStrides &,
                                                cudaStream_t);
template cudaError_t launch_simt_phase2<float>(const DevicePlan &, const float *, const float *,
                                               double *, float *, double, const RootStrides &,
                                               cudaStream_t);

} // namespace b2g
