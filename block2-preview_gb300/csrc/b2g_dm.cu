// Density-matrix truncation after a two-site step, FP64 on the device.
//
// Restates MovingEnvironment::density_matrix (src/dmrg/moving_environment.hpp:
// 3554-3580, through OperatorFunctions::trans_product,
// src/core/operator_functions.hpp:777-838, without noise),
// truncate_density_matrix (moving_environment.hpp:3715-3843, Physical
// truncation: keep the k largest eigenvalues, discarded weight = sum of the
// positive discarded ones, then drop trailing kept states below cutoff) and
// split_density_matrix (moving_environment.hpp:4250-4345: kept eigenvectors
// form the rotation tensor, the other tensor is rotation^T psi, normalised).
//
// Device work: rho blocks (batched SYRK, one thread per lower-triangle
// element), the Householder tridiagonalisation and orthogonal factor of every
// rho block (one CTA per block, a cluster of CTAs per large block), the
// application of the QL rotations to the eigenvector matrix, the gather of
// the kept eigenvectors and the split GEMMs.  Host work: the QL recurrence on
// each tridiagonal (a scalar chain of dependent FP64 operations, see below)
// and the selection of the kept states (a sort of at most a few thousand
// eigenvalues), in the reference's order.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

#include "b2g_internal.h"

namespace b2g {

namespace {

// rho_b[i][j] (j <= i, mirrored) = sum over psi blocks a of block b of
//   trace_right: sum_c psi_a[i][c] psi_a[j][c]     (rows of psi_a)
//   otherwise:   sum_r psi_a[r][i] psi_a[r][j]     (columns of psi_a)
__global__ void rho_kernel(const double *__restrict__ psi, const int32_t *__restrict__ list_ptr,
                           const int32_t *__restrict__ list, const int32_t *__restrict__ prow,
                           const int32_t *__restrict__ pcol, const uint64_t *__restrict__ poff,
                           const int32_t *__restrict__ dim, const uint64_t *__restrict__ rho_off,
                           double *__restrict__ rho, int trace_right) {
    const int b = blockIdx.y;
    const int n = dim[b];
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n * n)
        return;
    const int i = (int)(e / n), j = (int)(e % n);
    if (j > i)
        return;
    double s = 0.0;
    for (int q = list_ptr[b]; q < list_ptr[b + 1]; q++) {
        const int a = list[q];
        const double *P = psi + poff[a];
        const int r = prow[a], c = pcol[a];
        if (trace_right)
            for (int k = 0; k < c; k++)
                s = fma(P[(int64_t)i * c + k], P[(int64_t)j * c + k], s);
        else
            for (int k = 0; k < r; k++)
                s = fma(P[(int64_t)k * c + i], P[(int64_t)k * c + j], s);
    }
    rho[rho_off[b] + (int64_t)i * n + j] = s;
    rho[rho_off[b] + (int64_t)j * n + i] = s;
}

// Block-wide sum over kThreads threads (all threads get the result).
constexpr int kEigThreads = 256;
// The final sum over the warps is a pairwise tree (shallow FP64 dependency).
__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();  // red may still be read by a previous call
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    static_assert(kEigThreads / 32 == 8, "tree below sums 8 warps");
    return ((red[0] + red[1]) + (red[2] + red[3])) + ((red[4] + red[5]) + (red[6] + red[7]));
}


// Symmetric eigen-decomposition of the density-matrix blocks, FP64, as a
// GPU + host pipeline (the published Bowdler-Martin-Reinsch-Wilkinson method,
// the same reduction + QL family LAPACK's dsyev uses, ~9 n^3 flops):
//   1. device: Householder reduction of each block to tridiagonal (d, e) and
//      explicit accumulation of the orthogonal factor Q (stored transposed:
//      row i of Z is column i of Q) -- block-wide matrix-vector products and
//      rank-2 updates, one CTA per block or a cluster of CTAs per large block;
//   2. host: the implicit QL iteration with Wilkinson shifts on (d, e), which
//      is a scalar recurrence (each plane rotation depends on the previous
//      one): a dependent FP64 operation on GB300's narrow FP64 pipe costs ~100
//      cycles, on a Grace core a few, so the chase runs on the host cores
//      (blocks in parallel) and records its rotations;
//   3. device: the recorded rotations are applied to the rows of Z, every
//      column independently (one thread per column), giving the eigenvectors.
// Dynamic shared memory of the reduction kernels: 5 n doubles (d, e, beta, v, p).
constexpr int kQlMaxIter = 60;
constexpr int kDmMaxDim = 4000;  // 5 n doubles of shared memory stay below 227 KB
__global__ void __launch_bounds__(kEigThreads) eig_block(double *__restrict__ Aall,
                                                         double *__restrict__ Zall,
                                                         const int32_t *__restrict__ dim,
                                                         const uint64_t *__restrict__ off,
                                                         double *__restrict__ de_all,
                                                         const uint64_t *__restrict__ woff,
                                                         int skip_from) {
    extern __shared__ double sm[];
    __shared__ double red[kEigThreads / 32];
    const int b = blockIdx.x;
    const int n = dim[b];
    if (n == 0 || n >= skip_from)  // empty, or taken by eig_cluster
        return;
    double *A = Aall + off[b], *Z = Zall + off[b];
    double *d = sm, *e = sm + n, *beta = sm + 2 * n, *v = sm + 3 * n, *p = sm + 4 * n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int nwarps = kEigThreads / 32;

    // ---- 1. Householder reduction: step k zeroes A[k+2.., k]
    for (int k = 0; k + 2 < n; k++) {
        const int len = n - k - 1;
        const double *xk = A + (int64_t)k * n + k + 1;  // row k right of the diagonal
        double ss = 0.0;
        for (int i = tid; i < len; i += kEigThreads)
            ss += xk[i] * xk[i];
        const double sigma = block_sum(ss, red);
        const double x0 = xk[0];
        const double tail = sigma - x0 * x0;
        if (tid == 0)
            d[k] = A[(int64_t)k * n + k];
        if (tail <= 0.0) {  // already tridiagonal in this column
            if (tid == 0)
                e[k] = x0, beta[k] = 0.0;
            __syncthreads();
            continue;
        }
        const double alpha = x0 >= 0 ? -sqrt(sigma) : sqrt(sigma);
        const double bt = 1.0 / (sigma - x0 * alpha);
        for (int i = tid; i < len; i += kEigThreads)
            v[i] = i == 0 ? x0 - alpha : xk[i];
        __syncthreads();
        // p = beta * B v,  B = A[k+1.., k+1..]  (one warp per row)
        for (int i = warp; i < len; i += nwarps) {
            const double *Bi = A + (int64_t)(k + 1 + i) * n + k + 1;
            double acc = 0.0;
            for (int j = lane; j < len; j += 32)
                acc = fma(Bi[j], v[j], acc);
            for (int o = 16; o > 0; o >>= 1)
                acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0)
                p[i] = bt * acc;
        }
        __syncthreads();
        double vp = 0.0;
        for (int i = tid; i < len; i += kEigThreads)
            vp += v[i] * p[i];
        const double K = 0.5 * bt * block_sum(vp, red);
        for (int i = tid; i < len; i += kEigThreads)
            p[i] -= K * v[i];  // p <- w
        __syncthreads();
        // B <- B - v w^T - w v^T
        for (int i = warp; i < len; i += nwarps) {
            double *Bi = A + (int64_t)(k + 1 + i) * n + k + 1;
            const double vi = v[i], wi = p[i];
            for (int j = lane; j < len; j += 32)
                Bi[j] -= vi * p[j] + wi * v[j];
        }
        // keep the reflector in row k for the accumulation
        for (int i = tid; i < len; i += kEigThreads)
            A[(int64_t)k * n + k + 1 + i] = v[i];
        if (tid == 0)
            e[k] = alpha, beta[k] = bt;
        __syncthreads();
    }
    if (tid == 0) {
        if (n >= 2) {
            d[n - 2] = A[(int64_t)(n - 2) * n + n - 2];
            e[n - 2] = A[(int64_t)(n - 2) * n + n - 1];
        }
        d[n - 1] = A[(int64_t)(n - 1) * n + n - 1];
        e[n - 1] = 0.0;
    }
    // ---- 2. Q = H_0 H_1 ... H_{n-3}, built backwards, stored transposed in Z
    for (int64_t q = tid; q < (int64_t)n * n; q += kEigThreads)
        Z[q] = (q / n == q % n) ? 1.0 : 0.0;
    __syncthreads();
    for (int k = n - 3; k >= 0; k--) {
        const double bt = beta[k];
        if (bt == 0.0)
            continue;
        const int len = n - k - 1;
        for (int i = tid; i < len; i += kEigThreads)
            v[i] = A[(int64_t)k * n + k + 1 + i];
        __syncthreads();
        // y_i = sum_r v_r Q[r][i] = (row i of Z) . v ; then Z[i][r] -= beta y_i v_r
        for (int i = warp; i < len; i += nwarps) {
            const double *Zi = Z + (int64_t)(k + 1 + i) * n + k + 1;
            double acc = 0.0;
            for (int j = lane; j < len; j += 32)
                acc = fma(Zi[j], v[j], acc);
            for (int o = 16; o > 0; o >>= 1)
                acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0)
                p[i] = bt * acc;
        }
        __syncthreads();
        for (int i = warp; i < len; i += nwarps) {
            double *Zi = Z + (int64_t)(k + 1 + i) * n + k + 1;
            const double yi = p[i];
            for (int j = lane; j < len; j += 32)
                Zi[j] -= yi * v[j];
        }
        __syncthreads();
    }
    // ---- 3. the tridiagonal goes to the host (d, then e)
    __syncthreads();
    for (int i = tid; i < n; i += kEigThreads) {
        de_all[2 * woff[b] + i] = d[i];
        de_all[2 * woff[b] + n + i] = e[i];
    }
}

// ---- Large blocks: the reduction and Q accumulation on a cluster of
// kDmCluster CTAs (one SM each), so the FP64 pipes of kDmCluster SMs share one
// block.  Rows have fixed owners, row r on CTA r % kDmCluster; every CTA keeps
// its own copy of the tridiagonal and makes the same decisions from the same
// data.  Per reflector step two cluster barriers (the p vector and its dot
// product with v are exchanged through global scratch); the accumulation of Q
// is row-local (row i of Z changes with row i only) and needs none.  Data
// another CTA wrote is read with ld.global.cg (L2), behind the barrier's
// release/acquire and a __threadfence.
constexpr int kDmCluster = 8;
constexpr int kDmClusterMin = 96;  // blocks at least this large take the cluster path

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// every thread of every CTA of the cluster calls this at the same points
__device__ __forceinline__ void cluster_barrier() {
    __threadfence();
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// scratch per block (doubles): P[n] | VP[kDmCluster]
__host__ __device__ constexpr uint64_t dm_cluster_scratch(int n) { return (uint64_t)n + kDmCluster; }

__global__ void __cluster_dims__(kDmCluster, 1, 1) __launch_bounds__(kEigThreads)
    eig_cluster(double *__restrict__ Aall, double *__restrict__ Zall, const int32_t *__restrict__ dim,
                const uint64_t *__restrict__ off, double *__restrict__ de_all,
                const uint64_t *__restrict__ woff, const int32_t *__restrict__ big,
                double *__restrict__ scr_all, const uint64_t *__restrict__ scr_off) {
    extern __shared__ double sm[];
    __shared__ double red[kEigThreads / 32];
    const int rank = (int)cluster_rank();
    const int b = big[blockIdx.x / kDmCluster];
    const int n = dim[b];
    double *A = Aall + off[b], *Z = Zall + off[b];
    double *P = scr_all + scr_off[b], *VP = P + n;
    double *d = sm, *e = sm + n, *beta = sm + 2 * n, *v = sm + 3 * n, *p = sm + 4 * n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int nwarps = kEigThreads / 32, C = kDmCluster;
    // first row >= lo owned by this CTA
    auto first_own = [&](int lo) { return lo + ((rank - lo % C) % C + C) % C; };

    // ---- 1. Householder reduction (step k zeroes A[k+2.., k])
    for (int k = 0; k + 2 < n; k++) {
        const int len = n - k - 1;
        const double *xk = A + (int64_t)k * n + k + 1;
        double ss = 0.0;
        for (int i = tid; i < len; i += kEigThreads) {
            const double x = __ldcg(xk + i);
            ss += x * x;
        }
        const double sigma = block_sum(ss, red);
        const double x0 = __ldcg(xk);
        const double tail = sigma - x0 * x0;
        if (tid == 0)
            d[k] = __ldcg(A + (int64_t)k * n + k);
        if (tail <= 0.0) {  // same decision on every CTA
            if (tid == 0)
                e[k] = x0, beta[k] = 0.0;
            __syncthreads();
            continue;
        }
        const double alpha = x0 >= 0 ? -sqrt(sigma) : sqrt(sigma);
        const double bt = 1.0 / (sigma - x0 * alpha);
        for (int i = tid; i < len; i += kEigThreads)
            v[i] = i == 0 ? x0 - alpha : __ldcg(xk + i);
        __syncthreads();
        // p_i = beta B_i v for the owned rows r = k + 1 + i (one warp per row)
        double vpl = 0.0;
        for (int r = first_own(k + 1) + warp * C; r < n; r += C * nwarps) {
            const int i = r - k - 1;
            const double *Bi = A + (int64_t)r * n + k + 1;
            double acc = 0.0;
            for (int j = lane; j < len; j += 32)
                acc = fma(Bi[j], v[j], acc);
            for (int o = 16; o > 0; o >>= 1)
                acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) {
                P[i] = bt * acc;
                vpl += v[i] * (bt * acc);
            }
        }
        const double vps = block_sum(vpl, red);
        if (tid == 0)
            VP[rank] = vps;
        cluster_barrier();
        static_assert(kDmCluster == 8, "tree below sums 8 partials");
        double vq[kDmCluster];
#pragma unroll
        for (int c = 0; c < C; c++)
            vq[c] = __ldcg(VP + c);
        const double vp = ((vq[0] + vq[1]) + (vq[2] + vq[3])) + ((vq[4] + vq[5]) + (vq[6] + vq[7]));
        const double K = 0.5 * bt * vp;
        for (int i = tid; i < len; i += kEigThreads)
            p[i] = __ldcg(P + i) - K * v[i];  // p <- w
        __syncthreads();
        // B <- B - v w^T - w v^T on the owned rows
        for (int r = first_own(k + 1) + warp * C; r < n; r += C * nwarps) {
            const int i = r - k - 1;
            double *Bi = A + (int64_t)r * n + k + 1;
            const double vi = v[i], wi = p[i];
            for (int j = lane; j < len; j += 32)
                Bi[j] -= vi * p[j] + wi * v[j];
        }
        // the reflector replaces row k (its owner writes it)
        if (k % C == rank)
            for (int i = tid; i < len; i += kEigThreads)
                A[(int64_t)k * n + k + 1 + i] = v[i];
        if (tid == 0)
            e[k] = alpha, beta[k] = bt;
        cluster_barrier();
    }
    if (tid == 0) {
        d[n - 2] = __ldcg(A + (int64_t)(n - 2) * n + n - 2);
        e[n - 2] = __ldcg(A + (int64_t)(n - 2) * n + n - 1);
        d[n - 1] = __ldcg(A + (int64_t)(n - 1) * n + n - 1);
        e[n - 1] = 0.0;
    }
    // ---- 2. Q = H_0 H_1 ... H_{n-3}, built backwards, stored transposed in Z
    // (row i of Z = column i of Q); step k changes rows i >= k + 1, each alone
    for (int r = first_own(0) + warp * C; r < n; r += C * nwarps)
        for (int c = lane; c < n; c += 32)
            Z[(int64_t)r * n + c] = r == c ? 1.0 : 0.0;
    for (int k = n - 3; k >= 0; k--) {
        const double bt = beta[k];
        if (bt == 0.0)
            continue;
        const int len = n - k - 1;
        __syncthreads();
        for (int i = tid; i < len; i += kEigThreads)
            v[i] = __ldcg(A + (int64_t)k * n + k + 1 + i);
        __syncthreads();
        for (int r = first_own(k + 1) + warp * C; r < n; r += C * nwarps) {
            double *Zr = Z + (int64_t)r * n + k + 1;
            double acc = 0.0;
            for (int j = lane; j < len; j += 32)
                acc = fma(Zr[j], v[j], acc);
            for (int o = 16; o > 0; o >>= 1)
                acc += __shfl_xor_sync(0xffffffffu, acc, o);
            const double y = bt * acc;
            for (int j = lane; j < len; j += 32)
                Zr[j] -= y * v[j];
        }
    }
    // ---- 3. the tridiagonal goes to the host (d, then e)
    if (rank == 0) {
        __syncthreads();
        for (int i = tid; i < n; i += kEigThreads) {
            de_all[2 * woff[b] + i] = d[i];
            de_all[2 * woff[b] + n + i] = e[i];
        }
    }
}

// Applies the host-recorded QL rotations of every block to the rows of Z
// (Z = Q^T on entry, eigenvectors as rows on exit).  QL iteration it of block
// b acts on rows [m - cnt, m]: its rotation t (c, s) mixes rows m-1-t and m-t.
// Each column is independent: one thread per column, in iteration order.
__global__ void __launch_bounds__(64) apply_rotations(double *__restrict__ Zall,
                                                      const int32_t *__restrict__ dim,
                                                      const uint64_t *__restrict__ off,
                                                      const int64_t *__restrict__ it_first,
                                                      const int32_t *__restrict__ it_m,
                                                      const int32_t *__restrict__ it_cnt,
                                                      const int64_t *__restrict__ it_rot,
                                                      const double *__restrict__ rc,
                                                      const double *__restrict__ rs) {
    const int b = blockIdx.y, n = dim[b];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n)
        return;
    double *Z = Zall + off[b];
    for (int64_t it = it_first[b]; it < it_first[b + 1]; it++) {
        const int m = it_m[it], cnt = it_cnt[it];
        const double *cs = rc + it_rot[it], *sn = rs + it_rot[it];
        double carry = Z[(int64_t)m * n + r];
        double zn = Z[(int64_t)(m - 1) * n + r];
        for (int t = 0; t < cnt; t++) {
            const int i = m - 1 - t;
            const double zi = zn;
            if (t + 1 < cnt)
                zn = Z[(int64_t)(i - 1) * n + r];
            const double c = cs[t], sv = sn[t];
            Z[(int64_t)(i + 1) * n + r] = sv * zi + c * carry;
            carry = c * zi - sv * carry;
        }
        Z[(int64_t)(m - cnt) * n + r] = carry;
    }
}

// The same with the thread's column and each iteration's rotations staged in
// shared memory (one warp per CTA, 32 columns), the next rotation and row
// loaded one step ahead: the chain then waits on FP64 latency only, not on a
// global load per step.  Needs 272 n bytes; used for n <= 800.
constexpr int kRotSmemMaxDim = 800;
__global__ void __launch_bounds__(32) apply_rotations_smem(double *__restrict__ Zall,
                                                           const int32_t *__restrict__ dim,
                                                           const uint64_t *__restrict__ off,
                                                           const int64_t *__restrict__ it_first,
                                                           const int32_t *__restrict__ it_m,
                                                           const int32_t *__restrict__ it_cnt,
                                                           const int64_t *__restrict__ it_rot,
                                                           const double *__restrict__ rc,
                                                           const double *__restrict__ rs) {
    extern __shared__ double sz[];  // sz[i * 32 + lane] = Z[i][c0 + lane], then c[n], s[n]
    const int b = blockIdx.y, n = dim[b], lane = threadIdx.x;
    double *sc = sz + 32 * (size_t)n, *ss = sc + n;
    const int r = blockIdx.x * 32 + lane;
    if (blockIdx.x * 32 >= n)
        return;
    const bool live = r < n;
    double *Z = Zall + off[b];
    for (int i = 0; i < n; i++)
        sz[i * 32 + lane] = live ? Z[(int64_t)i * n + r] : 0.0;
    for (int64_t it = it_first[b]; it < it_first[b + 1]; it++) {
        const int m = it_m[it], cnt = it_cnt[it];
        const double *cs = rc + it_rot[it], *sn = rs + it_rot[it];
        __syncwarp();
        for (int t = lane; t < cnt; t += 32)
            sc[t] = cs[t], ss[t] = sn[t];
        __syncwarp();
        double carry = sz[m * 32 + lane];
        double zn = sz[(m - 1) * 32 + lane];
        double cn = sc[0], sn1 = ss[0];
        for (int t = 0; t < cnt; t++) {
            const int i = m - 1 - t;
            const double zi = zn, c = cn, sv = sn1;
            if (t + 1 < cnt)
                zn = sz[(i - 1) * 32 + lane], cn = sc[t + 1], sn1 = ss[t + 1];
            sz[(i + 1) * 32 + lane] = sv * zi + c * carry;
            carry = c * zi - sv * carry;
        }
        sz[(m - cnt) * 32 + lane] = carry;
    }
    if (live)
        for (int i = 0; i < n; i++)
            Z[(int64_t)i * n + r] = sz[i * 32 + lane];
}

// rotation blocks from the eigenvectors (rows of Z): for kept state q (global
// index, blocks in order, ascending eigenvalue within a block) of block b
// held in row ei of Z_b, trace_right: rot[rot_off[b] + r * im + j] = Z_b[ei][r],
// else rot[rot_off[b] + j * n + r] = Z_b[ei][r] (j = q - first kept of b)
__global__ void gather_rotation(double *__restrict__ rot, const double *__restrict__ Zall,
                                const int32_t *__restrict__ qb, const int32_t *__restrict__ qj,
                                const int32_t *__restrict__ qe, const int32_t *__restrict__ dim,
                                const int32_t *__restrict__ kept, const uint64_t *__restrict__ roff,
                                const uint64_t *__restrict__ rot_off, int n_kept, int trace_right) {
    const int q = blockIdx.x;
    if (q >= n_kept)
        return;
    const int b = qb[q], j = qj[q], ei = qe[q], n = dim[b], im = kept[b];
    const double *src = Zall + roff[b] + (uint64_t)ei * n;
    double *dst = rot + rot_off[b];
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        if (trace_right)
            dst[(uint64_t)r * im + j] = src[r];
        else
            dst[(uint64_t)j * n + r] = src[r];
    }
}

// The split GEMMs of all psi blocks in one launch: task a computes
// out_a (m x n) = op(X_a) (m x k) * op(Y_a) (k x n), row-major, FP64, one
// thread per element with four interleaved partial sums (shorter FP64
// dependency chains).
struct SplitTask {
    uint64_t out, x, y;       // offsets into the output, X and Y buffers
    int32_t ldx, tx, ldy, ty, m, n, k, pad;
};
__global__ void split_gemm(double *__restrict__ outb, const double *__restrict__ Xb,
                           const double *__restrict__ Yb, const SplitTask *__restrict__ tasks) {
    const SplitTask t = tasks[blockIdx.y];
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)t.m * t.n)
        return;
    const int i = (int)(e / t.n), j = (int)(e % t.n);
    const double *X = Xb + t.x, *Y = Yb + t.y;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int l = 0; l < t.k; l++) {
        const double x = t.tx ? X[(int64_t)l * t.ldx + i] : X[(int64_t)i * t.ldx + l];
        const double y = t.ty ? Y[(int64_t)j * t.ldy + l] : Y[(int64_t)l * t.ldy + j];
        s[l & 3] = fma(x, y, s[l & 3]);
    }
    outb[t.out + e] = (s[0] + s[1]) + (s[2] + s[3]);
}

// ---- host part of the eigensolver: implicit QL with Wilkinson shifts on the
// tridiagonal (d, e) of one block, e[i] coupling i and i+1 (e[n-1] = 0), with
// deflation against eps * max_i(|d_i| + |e_i|) (absolute accuracy, as
// LAPACK's; a local test never deflates the numerically-zero tail of a
// rank-deficient rho).  Records every iteration's plane rotations for
// apply_rotations.  Returns false if an eigenvalue needs more than
// kQlMaxIter iterations.
struct QlRecord {
    std::vector<int32_t> m, cnt;
    std::vector<int64_t> rot;  // first rotation of each iteration (block-local)
    std::vector<double> c, s;
};

bool ql_host(double *d, double *e, int n, QlRecord &rec) {
    double anorm = 0.0;
    for (int i = 0; i < n; i++)
        anorm = std::max(anorm, std::fabs(d[i]) + std::fabs(e[i]));
    const double tol = 2.220446049250313e-16 * anorm;
    int l = 0, iter = 0;
    while (l < n) {
        int m = l;
        for (; m < n - 1; m++)
            if (std::fabs(e[m]) <= tol)
                break;
        if (m == l) {
            l++, iter = 0;
            continue;
        }
        if (iter >= kQlMaxIter)
            return false;
        iter++;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        const double rr = std::hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0 ? rr : -rr));
        double s = 1.0, c = 1.0, pp = 0.0;
        const int64_t first = (int64_t)rec.c.size();
        bool underflow = false;
        for (int i = m - 1; i >= l; i--) {
            const double f = s * e[i], bb = c * e[i];
            const double h = std::fma(f, f, g * g);
            if (h == 0.0) {
                e[i + 1] = 0.0;
                d[i + 1] -= pp;
                e[m] = 0.0;
                underflow = true;
                break;
            }
            const double r = std::sqrt(h);
            e[i + 1] = r;
            s = f / r, c = g / r;
            g = d[i + 1] - pp;
            const double t = (d[i] - g) * s + 2.0 * c * bb;
            pp = s * t;
            d[i + 1] = g + pp;
            g = c * t - bb;
            rec.c.push_back(c), rec.s.push_back(s);
        }
        if (!underflow) {
            d[l] -= pp;
            e[l] = g;
            e[m] = 0.0;
        }
        const int cnt = (int)((int64_t)rec.c.size() - first);
        if (cnt > 0)
            rec.m.push_back(m), rec.cnt.push_back(cnt), rec.rot.push_back(first);
    }
    return true;
}

} // namespace

} // namespace b2g

using namespace b2g;

extern "C" int b2g_dm_truncate(b2g_context *ctx, const b2g_dm_layout *lay, const double *psi,
                               int k, double cutoff, double *eigvals, int32_t *kept,
                               double *rotation, double *wfn, b2g_dm_result *res) {
    if (ctx == nullptr || lay == nullptr || psi == nullptr || eigvals == nullptr || kept == nullptr ||
        rotation == nullptr || wfn == nullptr || res == nullptr)
        return fail(B2G_ERR_ARG, "b2g_dm_truncate: null argument");
    const int na = lay->n_psi_blocks, nb = lay->n_dm_blocks;
    if (na < 0 || nb < 0)
        return fail(B2G_ERR_ARG, "b2g_dm_truncate: negative block count");
    if (k < -1)
        return fail(B2G_ERR_ARG, "b2g_dm_truncate: k must be -1 (keep all) or non-negative");
    if (nb > 65535)
        return fail(B2G_ERR_UNSUPPORTED, "b2g_dm_truncate: more than 65535 density-matrix blocks");
    for (int b = 0; b < nb; b++)
        if (lay->dm_dim[b] > kDmMaxDim)
            return fail(B2G_ERR_UNSUPPORTED, "b2g_dm_truncate: density-matrix block above 4000 states");
    const bool tr = lay->trace_right != 0;
    // ---- host-side layout checks and tables
    uint64_t psi_size = 0, psi_sum = 0;
    std::vector<int32_t> lptr(nb + 1, 0), list;
    for (int a = 0; a < na; a++) {
        const int b = lay->psi_dm[a];
        if (lay->psi_rows[a] < 0 || lay->psi_cols[a] < 0)
            return fail(B2G_ERR_ARG, "b2g_dm_truncate: negative psi block size");
        psi_size = std::max<uint64_t>(psi_size, lay->psi_off[a] + (uint64_t)lay->psi_rows[a] * lay->psi_cols[a]);
        psi_sum += (uint64_t)lay->psi_rows[a] * lay->psi_cols[a];
        if (b < -1 || b >= nb)
            return fail(B2G_ERR_ARG, "b2g_dm_truncate: psi block maps to a missing dm block");
        if (b >= 0 && (tr ? lay->psi_rows[a] : lay->psi_cols[a]) != lay->dm_dim[b])
            return fail(B2G_ERR_ARG, "b2g_dm_truncate: psi block does not match its dm block size");
        if (b >= 0)
            lptr[b + 1]++;
    }
    if (psi_sum > psi_size)
        return fail(B2G_ERR_ARG, "b2g_dm_truncate: psi blocks overlap");
    for (int b = 0; b < nb; b++) {
        if (lay->dm_dim[b] < 0)
            return fail(B2G_ERR_ARG, "b2g_dm_truncate: negative density-matrix block size");
        lptr[b + 1] += lptr[b];
    }
    list.resize(lptr[nb]);
    {
        std::vector<int32_t> fill(lptr.begin(), lptr.end() - 1);
        for (int a = 0; a < na; a++)
            if (lay->psi_dm[a] >= 0)
                list[fill[lay->psi_dm[a]]++] = a;
    }
    std::vector<uint64_t> roff(nb), woff(nb);
    uint64_t rtot = 0, wtot = 0;
    int maxdim = 0;
    for (int b = 0; b < nb; b++) {
        roff[b] = rtot, woff[b] = wtot;
        rtot += (uint64_t)lay->dm_dim[b] * lay->dm_dim[b];
        wtot += (uint64_t)lay->dm_dim[b];
        maxdim = std::max(maxdim, lay->dm_dim[b]);
    }
    // blocks of at least kDmClusterMin states go to eig_cluster
    std::vector<int32_t> big;
    std::vector<uint64_t> scr_off(nb, 0);
    uint64_t scr_tot = 0;
    int maxbig = 0;
    for (int b = 0; b < nb; b++)
        if (lay->dm_dim[b] >= kDmClusterMin) {
            big.push_back(b);
            scr_off[b] = scr_tot;
            scr_tot += dm_cluster_scratch(lay->dm_dim[b]);
            maxbig = std::max(maxbig, lay->dm_dim[b]);
        }
    const int nbig = (int)big.size();
    B2G_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    // ---- device buffers: one arena, carved in 256-byte aligned pieces
    const size_t na1 = (size_t)std::max(na, 1), nb1 = (size_t)std::max(nb, 1);
    const uint64_t ksz = std::max<uint64_t>(wtot, 1);
    size_t arena = 0;
    auto take = [&](size_t bytes) {
        const size_t o = arena;
        arena += (bytes + 255) & ~(size_t)255;
        return o;
    };
    const size_t o_psi = take(sizeof(double) * std::max<uint64_t>(psi_size, 1));
    const size_t o_rho = take(sizeof(double) * std::max<uint64_t>(rtot, 1));
    const size_t o_z = take(sizeof(double) * std::max<uint64_t>(rtot, 1));
    const size_t o_de = take(sizeof(double) * 2 * ksz);
    const size_t o_rot = take(sizeof(double) * std::max<uint64_t>(rtot, 1));
    const size_t o_out = take(sizeof(double) * std::max<uint64_t>(psi_size, 1));
    const size_t o_scr = take(sizeof(double) * std::max<uint64_t>(scr_tot, 1));
    const size_t o_lptr = take(sizeof(int32_t) * (nb + 1));
    const size_t o_list = take(sizeof(int32_t) * std::max<size_t>(list.size(), 1));
    const size_t o_prow = take(sizeof(int32_t) * na1), o_pcol = take(sizeof(int32_t) * na1);
    const size_t o_dim = take(sizeof(int32_t) * nb1), o_kept = take(sizeof(int32_t) * nb1);
    const size_t o_big = take(sizeof(int32_t) * nb1);
    const size_t o_q = take(sizeof(int32_t) * 3 * ksz);
    const size_t o_poff = take(sizeof(uint64_t) * na1), o_roff = take(sizeof(uint64_t) * nb1);
    const size_t o_woff = take(sizeof(uint64_t) * nb1), o_scroff = take(sizeof(uint64_t) * nb1);
    const size_t o_rotoff = take(sizeof(uint64_t) * nb1), o_itf = take(sizeof(int64_t) * (nb + 1));
    const size_t o_tasks = take(sizeof(SplitTask) * na1);
    unsigned char *base = nullptr, *recs = nullptr;
    // stream-ordered pool allocations: freed without a device synchronisation
    // and reused by the next call
    if (cudaMallocAsync(&base, arena, s) != cudaSuccess)
        return fail(B2G_ERR_NOMEM, "b2g_dm_truncate: device allocation failed");
    double *d_psi = (double *)(base + o_psi), *d_rho = (double *)(base + o_rho);
    double *d_z = (double *)(base + o_z), *d_de = (double *)(base + o_de);
    double *d_rot = (double *)(base + o_rot), *d_out = (double *)(base + o_out);
    double *d_scr = (double *)(base + o_scr);
    int32_t *d_lptr = (int32_t *)(base + o_lptr), *d_list = (int32_t *)(base + o_list);
    int32_t *d_prow = (int32_t *)(base + o_prow), *d_pcol = (int32_t *)(base + o_pcol);
    int32_t *d_dim = (int32_t *)(base + o_dim), *d_kept = (int32_t *)(base + o_kept);
    int32_t *d_big = (int32_t *)(base + o_big), *d_q = (int32_t *)(base + o_q);
    uint64_t *d_poff = (uint64_t *)(base + o_poff), *d_roff = (uint64_t *)(base + o_roff);
    uint64_t *d_woff = (uint64_t *)(base + o_woff), *d_scroff = (uint64_t *)(base + o_scroff);
    uint64_t *d_rotoff = (uint64_t *)(base + o_rotoff);
    int64_t *d_itf = (int64_t *)(base + o_itf);
    SplitTask *d_tasks = (SplitTask *)(base + o_tasks);
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev_rho = nullptr, ev_small = nullptr;
    auto cleanup = [&]() {
        if (ev_rho) cudaEventDestroy(ev_rho);
        if (ev_small) cudaEventDestroy(ev_small);
        if (s2) cudaStreamDestroy(s2);
        cudaFreeAsync(base, s);
        if (recs)
            cudaFreeAsync(recs, s);
    };
    int rc = B2G_OK;
#define DM_TRY(expr)                                                                        \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess) {                                                            \
            rc = fail(B2G_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));    \
            goto done;                                                                      \
        }                                                                                   \
    } while (0)
    {
        DM_TRY(cudaMemcpyAsync(d_psi, psi, sizeof(double) * psi_size, cudaMemcpyHostToDevice, s));
        DM_TRY(cudaMemcpyAsync(d_lptr, lptr.data(), sizeof(int32_t) * (nb + 1), cudaMemcpyHostToDevice, s));
        if (!list.empty())
            DM_TRY(cudaMemcpyAsync(d_list, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice, s));
        if (na) {
            DM_TRY(cudaMemcpyAsync(d_prow, lay->psi_rows, sizeof(int32_t) * na, cudaMemcpyHostToDevice, s));
            DM_TRY(cudaMemcpyAsync(d_pcol, lay->psi_cols, sizeof(int32_t) * na, cudaMemcpyHostToDevice, s));
            DM_TRY(cudaMemcpyAsync(d_poff, lay->psi_off, sizeof(uint64_t) * na, cudaMemcpyHostToDevice, s));
        }
        if (nb) {
            DM_TRY(cudaMemcpyAsync(d_dim, lay->dm_dim, sizeof(int32_t) * nb, cudaMemcpyHostToDevice, s));
            DM_TRY(cudaMemcpyAsync(d_roff, roff.data(), sizeof(uint64_t) * nb, cudaMemcpyHostToDevice, s));
            DM_TRY(cudaMemcpyAsync(d_woff, woff.data(), sizeof(uint64_t) * nb, cudaMemcpyHostToDevice, s));
            DM_TRY(cudaMemcpyAsync(d_scroff, scr_off.data(), sizeof(uint64_t) * nb, cudaMemcpyHostToDevice, s));
        }
        if (nbig)
            DM_TRY(cudaMemcpyAsync(d_big, big.data(), sizeof(int32_t) * nbig, cudaMemcpyHostToDevice, s));
        std::vector<double> de(2 * wtot);
        if (nb && maxdim > 0) {
            const int64_t cells = (int64_t)maxdim * maxdim;
            note_launch();
            rho_kernel<<<dim3((unsigned)((cells + 255) / 256), nb), 256, 0, s>>>(
                d_psi, d_lptr, d_list, d_prow, d_pcol, d_poff, d_dim, d_roff, d_rho, tr ? 1 : 0);
            DM_TRY(cudaGetLastError());
            // small blocks (one CTA each) on a side stream, large blocks (one
            // cluster each) on the context stream, concurrently
            DM_TRY(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
            DM_TRY(cudaEventCreateWithFlags(&ev_rho, cudaEventDisableTiming));
            DM_TRY(cudaEventCreateWithFlags(&ev_small, cudaEventDisableTiming));
            DM_TRY(cudaEventRecord(ev_rho, s));
            DM_TRY(cudaStreamWaitEvent(s2, ev_rho, 0));
            const size_t smem = sizeof(double) * 5 * (size_t)maxdim;
            DM_TRY(cudaFuncSetAttribute(eig_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            note_launch();
            eig_block<<<nb, kEigThreads, smem, s2>>>(d_rho, d_z, d_dim, d_roff, d_de, d_woff,
                                                      nbig ? kDmClusterMin : kDmMaxDim + 1);
            DM_TRY(cudaGetLastError());
            DM_TRY(cudaEventRecord(ev_small, s2));
            if (nbig) {
                const size_t smem_c = sizeof(double) * 5 * (size_t)maxbig;
                DM_TRY(cudaFuncSetAttribute(eig_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem_c));
                note_launch();
                eig_cluster<<<kDmCluster * nbig, kEigThreads, smem_c, s>>>(d_rho, d_z, d_dim, d_roff, d_de,
                                                                          d_woff, d_big, d_scr, d_scroff);
                DM_TRY(cudaGetLastError());
            }
            DM_TRY(cudaStreamWaitEvent(s, ev_small, 0));
            DM_TRY(cudaMemcpyAsync(de.data(), d_de, sizeof(double) * 2 * wtot, cudaMemcpyDeviceToHost, s));
            DM_TRY(cudaStreamSynchronize(s));
        }
        // ---- host QL on every block (largest first over a few threads)
        std::vector<QlRecord> recs_h(nb);
        std::vector<char> ok(nb, 1);
        {
            std::vector<int> order(nb);
            std::iota(order.begin(), order.end(), 0);
            std::stable_sort(order.begin(), order.end(),
                             [&](int x, int y) { return lay->dm_dim[x] > lay->dm_dim[y]; });
            std::atomic<int> next{0};
            auto worker = [&]() {
                for (int t = next++; t < nb; t = next++) {
                    const int b = order[t], n = lay->dm_dim[b];
                    if (n > 0)
                        ok[b] = ql_host(de.data() + 2 * woff[b], de.data() + 2 * woff[b] + n, n, recs_h[b]);
                }
            };
            const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
            const int nth = (int)std::min<unsigned>(std::min<unsigned>(hw, 16u), (unsigned)std::max(nb, 1));
            std::vector<std::thread> pool;
            for (int t = 1; t < nth; t++)
                pool.emplace_back(worker);
            worker();
            for (auto &th : pool)
                th.join();
        }
        for (int b = 0; b < nb; b++)
            if (!ok[b]) {
                rc = fail(B2G_ERR_NOT_CONVERGED, "b2g_dm_truncate: QL iteration did not converge");
                goto done;
            }
        // ---- the rotations go back to the device and turn Z into eigenvectors
        {
            std::vector<int64_t> itf(nb + 1, 0), it_rot;
            std::vector<int32_t> it_m, it_cnt;
            std::vector<double> rcv, rsv;
            for (int b = 0; b < nb; b++) {
                const QlRecord &r = recs_h[b];
                itf[b] = (int64_t)it_m.size();
                for (size_t t = 0; t < r.m.size(); t++) {
                    it_m.push_back(r.m[t]), it_cnt.push_back(r.cnt[t]);
                    it_rot.push_back((int64_t)rcv.size() + r.rot[t]);
                }
                rcv.insert(rcv.end(), r.c.begin(), r.c.end());
                rsv.insert(rsv.end(), r.s.begin(), r.s.end());
            }
            itf[nb] = (int64_t)it_m.size();
            const size_t nit = std::max<size_t>(it_m.size(), 1), nrot = std::max<size_t>(rcv.size(), 1);
            const size_t r0 = 0, r1 = r0 + ((sizeof(int64_t) * nit + 255) & ~(size_t)255);
            const size_t r2 = r1 + ((sizeof(int32_t) * nit + 255) & ~(size_t)255);
            const size_t r3 = r2 + ((sizeof(int32_t) * nit + 255) & ~(size_t)255);
            const size_t r4 = r3 + ((sizeof(double) * nrot + 255) & ~(size_t)255);
            const size_t rend = r4 + sizeof(double) * nrot;
            if (cudaMallocAsync(&recs, rend, s) != cudaSuccess) {
                recs = nullptr;
                rc = fail(B2G_ERR_NOMEM, "b2g_dm_truncate: rotation record allocation failed");
                goto done;
            }
            DM_TRY(cudaMemcpyAsync(d_itf, itf.data(), sizeof(int64_t) * (nb + 1), cudaMemcpyHostToDevice, s));
            if (!it_m.empty()) {
                DM_TRY(cudaMemcpyAsync(recs + r0, it_rot.data(), sizeof(int64_t) * it_m.size(), cudaMemcpyHostToDevice, s));
                DM_TRY(cudaMemcpyAsync(recs + r1, it_m.data(), sizeof(int32_t) * it_m.size(), cudaMemcpyHostToDevice, s));
                DM_TRY(cudaMemcpyAsync(recs + r2, it_cnt.data(), sizeof(int32_t) * it_m.size(), cudaMemcpyHostToDevice, s));
                DM_TRY(cudaMemcpyAsync(recs + r3, rcv.data(), sizeof(double) * rcv.size(), cudaMemcpyHostToDevice, s));
                DM_TRY(cudaMemcpyAsync(recs + r4, rsv.data(), sizeof(double) * rsv.size(), cudaMemcpyHostToDevice, s));
            }
            if (nb && maxdim > 0 && maxdim <= kRotSmemMaxDim) {
                const size_t smem_r = sizeof(double) * 34 * (size_t)maxdim;
                DM_TRY(cudaFuncSetAttribute(apply_rotations_smem, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem_r));
                note_launch();
                apply_rotations_smem<<<dim3((unsigned)((maxdim + 31) / 32), nb), 32, smem_r, s>>>(
                    d_z, d_dim, d_roff, d_itf, (const int32_t *)(recs + r1), (const int32_t *)(recs + r2),
                    (const int64_t *)(recs + r0), (const double *)(recs + r3), (const double *)(recs + r4));
                DM_TRY(cudaGetLastError());
            } else if (nb && maxdim > 0) {
                note_launch();
                apply_rotations<<<dim3((unsigned)((maxdim + 63) / 64), nb), 64, 0, s>>>(
                    d_z, d_dim, d_roff, d_itf, (const int32_t *)(recs + r1), (const int32_t *)(recs + r2),
                    (const int64_t *)(recs + r0), (const double *)(recs + r3), (const double *)(recs + r4));
                DM_TRY(cudaGetLastError());
            }
        }
        // ---- eigenvalues ascending per block (perm: ascending position -> row of Z)
        std::vector<double> w(wtot);
        std::vector<int32_t> perm(wtot);
        for (int b = 0; b < nb; b++) {
            const int n = lay->dm_dim[b];
            const double *dd = de.data() + 2 * woff[b];
            int32_t *pb = perm.data() + woff[b];
            std::iota(pb, pb + n, 0);
            std::stable_sort(pb, pb + n, [&](int32_t x, int32_t y) { return dd[x] < dd[y]; });
            for (int j = 0; j < n; j++)
                w[woff[b] + j] = dd[pb[j]];
        }
        memcpy(eigvals, w.data(), sizeof(double) * wtot);
        // ---- selection, in the reference's order (truncate_density_matrix, Physical)
        std::vector<std::pair<int, int>> ss;
        for (int b = 0; b < nb; b++)
            for (int j = 0; j < lay->dm_dim[b]; j++)
                ss.push_back({b, j});
        const int k_total = (int)ss.size();
        double error = 0.0;
        auto ev = [&](const std::pair<int, int> &p) { return w[woff[p.first] + p.second]; };
        if (k >= 0) {
            std::sort(ss.begin(), ss.end(), [&](const std::pair<int, int> &x, const std::pair<int, int> &y) {
                return ev(x) > ev(y);
            });
            for (int i = k; i < k_total; i++)
                if (ev(ss[i]) > 0)
                    error += ev(ss[i]);
            int kk = std::min(k, k_total);
            for (; kk > 1 && ev(ss[kk - 1]) < cutoff; kk--)
                if (ev(ss[kk - 1]) > 0)
                    error += ev(ss[kk - 1]);
            if (kk < k_total)
                ss.resize(kk);
            std::sort(ss.begin(), ss.end());
        }
        std::fill(kept, kept + nb, 0);
        for (auto &p : ss)
            kept[p.first]++;
        res->error = error;
        res->n_kept = (int32_t)ss.size();
        // ---- rotation blocks on the device: kept eigenvectors, ascending eigen index
        //   trace_right: (dim x im), column j = eigenvector;  else (im x dim), row j = eigenvector
        std::vector<uint64_t> rot_off(nb);
        uint64_t rot_tot = 0;
        for (int b = 0; b < nb; b++) {
            rot_off[b] = rot_tot;
            rot_tot += (uint64_t)lay->dm_dim[b] * kept[b];
        }
        const int nk = (int)ss.size();
        if (nk > 0) {
            std::vector<int32_t> q(3 * (size_t)nk);
            for (int i = 0, j = 0; i < nk; i++) {
                j = (i > 0 && ss[i].first == ss[i - 1].first) ? j + 1 : 0;
                q[i] = ss[i].first, q[nk + i] = j;
                q[2 * nk + i] = perm[woff[ss[i].first] + ss[i].second];
            }
            DM_TRY(cudaMemcpyAsync(d_q, q.data(), sizeof(int32_t) * 3 * nk, cudaMemcpyHostToDevice, s));
            DM_TRY(cudaMemcpyAsync(d_kept, kept, sizeof(int32_t) * nb, cudaMemcpyHostToDevice, s));
            DM_TRY(cudaMemcpyAsync(d_rotoff, rot_off.data(), sizeof(uint64_t) * nb, cudaMemcpyHostToDevice, s));
            note_launch();
            gather_rotation<<<nk, 256, 0, s>>>(d_rot, d_z, d_q, d_q + nk, d_q + 2 * nk, d_dim, d_kept, d_roff,
                                               d_rotoff, nk, tr ? 1 : 0);
            DM_TRY(cudaGetLastError());
            DM_TRY(cudaMemcpyAsync(rotation, d_rot, sizeof(double) * rot_tot, cudaMemcpyDeviceToHost, s));
        }
        // ---- the other tensor: per psi block with kept states, normalised overall
        //   trace_right: rot_b^T (im x rows) psi_a (rows x cols);  else psi_a (rows x cols) rot_b^T (cols x im)
        uint64_t wpos = 0;
        std::vector<SplitTask> tasks;
        int64_t max_el = 0;
        for (int a = 0; a < na; a++) {
            const int b = lay->psi_dm[a];
            if (b < 0 || kept[b] == 0)
                continue;
            const int r = lay->psi_rows[a], c = lay->psi_cols[a], im = kept[b];
            if ((uint64_t)r * c == 0)
                continue;
            SplitTask t;
            t.out = wpos, t.pad = 0;
            if (tr) {  // rot_b^T (im x r) psi_a (r x c)
                t.x = rot_off[b], t.ldx = im, t.tx = 1, t.y = lay->psi_off[a], t.ldy = c, t.ty = 0;
                t.m = im, t.n = c, t.k = r;
            } else {   // psi_a (r x c) rot_b^T (c x im)
                t.x = lay->psi_off[a], t.ldx = c, t.tx = 0, t.y = rot_off[b], t.ldy = lay->dm_dim[b], t.ty = 1;
                t.m = r, t.n = im, t.k = c;
            }
            tasks.push_back(t);
            max_el = std::max<int64_t>(max_el, (int64_t)t.m * t.n);
            wpos += (uint64_t)t.m * t.n;
        }
        if (!tasks.empty()) {
            DM_TRY(cudaMemcpyAsync(d_tasks, tasks.data(), sizeof(SplitTask) * tasks.size(), cudaMemcpyHostToDevice, s));
            const double *xb = tr ? d_rot : d_psi, *yb = tr ? d_psi : d_rot;
            note_launch();
            split_gemm<<<dim3((unsigned)((max_el + 255) / 256), (unsigned)tasks.size()), 256, 0, s>>>(
                d_out, xb, yb, d_tasks);
            DM_TRY(cudaGetLastError());
        }
        std::vector<double> out(wpos);
        if (wpos)
            DM_TRY(cudaMemcpyAsync(out.data(), d_out, sizeof(double) * wpos, cudaMemcpyDeviceToHost, s));
        DM_TRY(cudaStreamSynchronize(s));
        double nrm = 0.0;
        for (double x : out)
            nrm += x * x;
        nrm = std::sqrt(nrm);
        for (uint64_t i = 0; i < wpos; i++)
            wfn[i] = nrm > 0 ? out[i] / nrm : 0.0;
    }
done:
#undef DM_TRY
    cudaStreamSynchronize(s);
    cleanup();
    return rc;
}
