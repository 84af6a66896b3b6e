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
// element), the symmetric eigen-decomposition of every rho block (one CTA
// per block: Householder tridiagonalisation + implicit QL, matrices in
// global memory, vectors in shared memory), and the split GEMMs.  The selection of the kept states (a sort of at most a few thousand
// eigenvalues) runs on the host, in the reference's order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
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
__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();  // red may still be read by a previous call
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int k = 0; k < kEigThreads / 32; k++)
        s += red[k];
    return s;
}

// Symmetric eigen-decomposition of one density-matrix block per CTA, FP64:
// Householder reduction to tridiagonal form, explicit accumulation of the
// orthogonal factor, then the implicit QL iteration with Wilkinson shifts on
// the tridiagonal (the published Bowdler-Martin-Reinsch-Wilkinson method, the
// same reduction + QL family LAPACK's dsyev uses).  The FP64 pipe of an SM is
// narrow, so the work is kept near the 9 n^3 flops of this method (a cyclic
// Jacobi needs ~60 n^3).  Parallel structure: the reflector steps are
// block-wide matrix-vector products and rank-2 updates; each QL iteration's
// rotation chase is a short scalar recurrence (one thread) whose rotations
// are then applied to all n rows of the eigenvector matrix in parallel.
//
// A: the block (n x n row-major, symmetric; overwritten by the reflectors).
// Z: scratch n x n, holds Z^T (row i = eigenvector i before sorting).
// V: out, row j = eigenvector of the j-th smallest eigenvalue (the storage
//    LAPACK leaves in a row-major matrix).  w: out, eigenvalues ascending.
// Dynamic shared memory: 7 n doubles (d, e, beta, v, p, rotation c, s;
// the QL phase reuses beta..s as two rotation slots).
constexpr int kQlMaxIter = 60;
constexpr int kConsumerWarps = kEigThreads / 32 - kEigThreads / 128;  // warps with (warp & 3) != 0

// The next QL iteration of the tridiagonal (d, e) (e[i] couples i and i+1):
// finds the unreduced block [l, m] (|e| <= tol splits), applies one implicit
// QL step with the Wilkinson shift from its top and records its plane
// rotations (c, s) in rc/rs in the order they are generated (pair m-1-t,
// m-t for rotation t).  state = {l, iterations spent on l}.  Returns false
// when every eigenvalue has converged.  Rotations use one rsqrt instead of a
// hypot and two divisions (|rho| stays far from the FP64 range limits).
__device__ __forceinline__ bool ql_next(double *d, double *e, int n, double tol, int *state, double *rc,
                        double *rs, int &m_out, int &cnt_out, int *err) {
    int l = state[0], iter = state[1];
    bool produced = false;
    while (l < n && !produced) {
        int m = l;
        for (; m < n - 1; m++)
            if (fabs(e[m]) <= tol)
                break;
        if (m == l) {
            l++, iter = 0;
            continue;
        }
        if (iter >= kQlMaxIter) {  // no convergence: flag it and leave this eigenvalue
            atomicExch(err, 2);
            l++, iter = 0;
            continue;
        }
        iter++;
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        const double rr = hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0 ? rr : -rr));
        double s = 1.0, c = 1.0, pp = 0.0;
        int cnt = 0;
        bool underflow = false;
        for (int i = m - 1; i >= l; i--) {
            const double f = s * e[i], bb = c * e[i];
            const double h = fma(f, f, g * g);
            if (h == 0.0) {
                e[i + 1] = 0.0;
                d[i + 1] -= pp;
                e[m] = 0.0;
                underflow = true;
                break;
            }
            const double inv = rsqrt(h);
            e[i + 1] = h * inv;
            s = f * inv, c = g * inv;
            g = d[i + 1] - pp;
            const double r = (d[i] - g) * s + 2.0 * c * bb;
            pp = s * r;
            d[i + 1] = g + pp;
            g = c * r - bb;
            rc[cnt] = c, rs[cnt] = s, cnt++;
        }
        if (!underflow) {
            d[l] -= pp;
            e[l] = g;
            e[m] = 0.0;
        }
        if (cnt > 0) {
            m_out = m, cnt_out = cnt;
            produced = true;
        }
    }
    state[0] = l, state[1] = iter;
    return produced;
}
constexpr int kDmMaxDim = 4000;  // 7 n doubles of shared memory stay below 227 KB
__global__ void __launch_bounds__(kEigThreads) eig_block(double *__restrict__ Aall,
                                                         double *__restrict__ Zall,
                                                         double *__restrict__ Vall,
                                                         const int32_t *__restrict__ dim,
                                                         const uint64_t *__restrict__ off,
                                                         double *__restrict__ wall,
                                                         const uint64_t *__restrict__ woff,
                                                         int *__restrict__ perm_all, int *err) {
    extern __shared__ double sm[];
    __shared__ double red[kEigThreads / 32];
    __shared__ int item_m[2], item_cnt[2], ql_state[2];
    __shared__ double ql_tol;
    const int b = blockIdx.x;
    const int n = dim[b];
    if (n == 0)
        return;
    double *A = Aall + off[b], *Z = Zall + off[b], *V = Vall + off[b], *w = wall + woff[b];
    int *perm = perm_all + woff[b] + b;
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
    // ---- 3. implicit QL with Wilkinson shifts on (d, e), two-stage pipeline:
    // thread 0 chases QL iteration t+1 (a scalar recurrence producing its
    // plane rotations) while warps 1.. apply the rotations of iteration t to
    // the rows of Z; one barrier per iteration.  Rotation slots reuse the
    // reflector scratch: slot s holds c at sm + (2 + 2s) n and s at + n.
    if (tid == 0) {
        // Deflation is tested against the norm of the whole tridiagonal
        // (absolute accuracy eps * |rho|, as LAPACK's): a local test never
        // deflates the numerically-zero tail of a rank-deficient rho.
        double anorm = 0.0;
        for (int i = 0; i < n; i++)
            anorm = fmax(anorm, fabs(d[i]) + fabs(e[i]));
        ql_state[0] = 0, ql_state[1] = 0;
        ql_tol = 2.220446049250313e-16 * anorm;
        int m = -1, cnt = 0;
        if (!ql_next(d, e, n, ql_tol, ql_state, sm + 2 * n, sm + 3 * n, m, cnt, err))
            m = -1;
        item_m[0] = m, item_cnt[0] = cnt;
    }
    __syncthreads();
    for (int t = 0;; t++) {  // at most kQlMaxIter * n items
        const int cur = t & 1;
        const int m = item_m[cur], cnt = item_cnt[cur];
        if (m < 0)
            break;
        if (tid == 0) {
            const int nx = cur ^ 1;
            int m2 = -1, cnt2 = 0;
            if (!ql_next(d, e, n, ql_tol, ql_state, sm + (2 + 2 * nx) * n, sm + (3 + 2 * nx) * n, m2,
                         cnt2, err))
                m2 = -1;
            item_m[nx] = m2, item_cnt[nx] = cnt2;
        } else if ((warp & 3) != 0) {
            // The consumers are the warps off thread 0's SM sub-partition, so
            // the chase keeps that sub-partition's FP64 pipe to itself.
            // Rotation t2 acts on eigenvector pair (m-1-t2, m-t2).
            const double *cs = sm + (2 + 2 * cur) * n, *sn = cs + n;
            const int cw = warp - 1 - (warp >> 2);  // 0 .. kConsumerWarps-1
            for (int r = cw * 32 + lane; r < n; r += kConsumerWarps * 32) {
                double carry = Z[(int64_t)m * n + r];
                double zn = Z[(int64_t)(m - 1) * n + r];
                for (int t2 = 0; t2 < cnt; t2++) {
                    const int i = m - 1 - t2;
                    const double zi = zn;
                    if (t2 + 1 < cnt)
                        zn = Z[(int64_t)(i - 1) * n + r];
                    const double c = cs[t2], sv = sn[t2];
                    Z[(int64_t)(i + 1) * n + r] = sv * zi + c * carry;
                    carry = c * zi - sv * carry;
                }
                Z[(int64_t)(m - cnt) * n + r] = carry;
            }
        }
        __syncthreads();
    }
    // ---- 4. ascending order (a stable selection on one thread; n is small)
    if (tid == 0) {
        for (int i = 0; i < n; i++)
            perm[i] = i;
        for (int i = 0; i < n; i++) {
            int bi = i;
            for (int j = i + 1; j < n; j++)
                if (d[perm[j]] < d[perm[bi]])
                    bi = j;
            const int t = perm[bi];
            for (int j = bi; j > i; j--)
                perm[j] = perm[j - 1];
            perm[i] = t;
        }
        for (int i = 0; i < n; i++)
            w[i] = d[perm[i]];
    }
    __syncthreads();
    for (int64_t q = tid; q < (int64_t)n * n; q += kEigThreads) {
        const int j = (int)(q / n), r = (int)(q % n);
        V[q] = Z[(int64_t)perm[j] * n + r];
    }
}

// out (m x n) = op(X) (m x k) * op(Y) (k x n), row-major, FP64, one thread per element
__global__ void small_gemm(double *__restrict__ out, const double *__restrict__ X, int ldx, int tx,
                           const double *__restrict__ Y, int ldy, int ty, int m, int n, int k) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)m * n)
        return;
    const int i = (int)(e / n), j = (int)(e % n);
    double s = 0.0;
    for (int l = 0; l < k; l++) {
        const double x = tx ? X[(int64_t)l * ldx + i] : X[(int64_t)i * ldx + l];
        const double y = ty ? Y[(int64_t)j * ldy + l] : Y[(int64_t)l * ldy + j];
        s = fma(x, y, s);
    }
    out[e] = s;
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
    B2G_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    // ---- device buffers
    double *d_psi = nullptr, *d_rho = nullptr, *d_vt = nullptr, *d_v = nullptr, *d_w = nullptr,
           *d_rot = nullptr, *d_out = nullptr;
    int32_t *d_lptr = nullptr, *d_list = nullptr, *d_prow = nullptr, *d_pcol = nullptr, *d_dim = nullptr;
    uint64_t *d_poff = nullptr, *d_roff = nullptr, *d_woff = nullptr;
    int *d_perm = nullptr, *d_err = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_psi), cudaFree(d_rho), cudaFree(d_vt), cudaFree(d_v), cudaFree(d_w);
        cudaFree(d_rot), cudaFree(d_out), cudaFree(d_lptr), cudaFree(d_list), cudaFree(d_prow);
        cudaFree(d_pcol), cudaFree(d_dim), cudaFree(d_poff), cudaFree(d_roff), cudaFree(d_woff);
        cudaFree(d_perm), cudaFree(d_err);
    };
    const size_t rb = sizeof(double) * std::max<uint64_t>(rtot, 1);
    if (cudaMalloc(&d_psi, sizeof(double) * std::max<uint64_t>(psi_size, 1)) ||
        cudaMalloc(&d_rho, rb) || cudaMalloc(&d_vt, rb) || cudaMalloc(&d_v, rb) ||
        cudaMalloc(&d_w, sizeof(double) * std::max<uint64_t>(wtot, 1)) ||
        cudaMalloc(&d_rot, rb) || cudaMalloc(&d_out, sizeof(double) * std::max<uint64_t>(psi_size, 1)) ||
        cudaMalloc(&d_lptr, sizeof(int32_t) * (nb + 1)) ||
        cudaMalloc(&d_list, sizeof(int32_t) * std::max<size_t>(list.size(), 1)) ||
        cudaMalloc(&d_prow, sizeof(int32_t) * std::max(na, 1)) ||
        cudaMalloc(&d_pcol, sizeof(int32_t) * std::max(na, 1)) ||
        cudaMalloc(&d_dim, sizeof(int32_t) * std::max(nb, 1)) ||
        cudaMalloc(&d_poff, sizeof(uint64_t) * std::max(na, 1)) ||
        cudaMalloc(&d_roff, sizeof(uint64_t) * std::max(nb, 1)) ||
        cudaMalloc(&d_woff, sizeof(uint64_t) * std::max(nb, 1)) ||
        cudaMalloc(&d_perm, sizeof(int) * (wtot + nb + 2)) || cudaMalloc(&d_err, sizeof(int))) {
        cleanup();
        return fail(B2G_ERR_NOMEM, "b2g_dm_truncate: device allocation failed");
    }
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
        }
        DM_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), s));
        if (nb && maxdim > 0) {
            const int64_t cells = (int64_t)maxdim * maxdim;
            rho_kernel<<<dim3((unsigned)((cells + 255) / 256), nb), 256, 0, s>>>(
                d_psi, d_lptr, d_list, d_prow, d_pcol, d_poff, d_dim, d_roff, d_rho, tr ? 1 : 0);
            DM_TRY(cudaGetLastError());
            const size_t smem = sizeof(double) * 7 * (size_t)maxdim;
            DM_TRY(cudaFuncSetAttribute(eig_block, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            eig_block<<<nb, kEigThreads, smem, s>>>(d_rho, d_vt, d_v, d_dim, d_roff, d_w, d_woff, d_perm, d_err);
            DM_TRY(cudaGetLastError());
        }
        std::vector<double> w(wtot);
        int errflag = 0;
        DM_TRY(cudaMemcpyAsync(w.data(), d_w, sizeof(double) * wtot, cudaMemcpyDeviceToHost, s));
        DM_TRY(cudaMemcpyAsync(&errflag, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        DM_TRY(cudaStreamSynchronize(s));
        if (errflag) {
            rc = fail(B2G_ERR_NOT_CONVERGED, "b2g_dm_truncate: QL iteration did not converge");
            goto done;
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
        // ---- rotation blocks: kept eigenvectors, ascending eigen index
        //   trace_right: (dim x im), column j = eigenvector;  else (im x dim), row j = eigenvector
        std::vector<double> V(rtot);
        DM_TRY(cudaMemcpyAsync(V.data(), d_v, sizeof(double) * rtot, cudaMemcpyDeviceToHost, s));
        DM_TRY(cudaStreamSynchronize(s));
        std::vector<uint64_t> rot_off(nb);
        std::vector<double> rot;
        {
            size_t iss = 0;
            for (int b = 0; b < nb; b++) {
                const int n = lay->dm_dim[b], im = kept[b];
                rot_off[b] = rot.size();
                std::vector<double> blk((size_t)n * im);
                for (int j = 0; j < im; j++) {
                    const int ei = ss[iss + j].second;
                    for (int r = 0; r < n; r++) {
                        const double v = V[roff[b] + (uint64_t)ei * n + r];
                        if (tr)
                            blk[(size_t)r * im + j] = v;
                        else
                            blk[(size_t)j * n + r] = v;
                    }
                }
                iss += im;
                rot.insert(rot.end(), blk.begin(), blk.end());
            }
        }
        if (!rot.empty()) {
            memcpy(rotation, rot.data(), sizeof(double) * rot.size());
            DM_TRY(cudaMemcpyAsync(d_rot, rot.data(), sizeof(double) * rot.size(), cudaMemcpyHostToDevice, s));
        }
        // ---- the other tensor: per psi block with kept states, normalised overall
        //   trace_right: rot_b^T (im x rows) psi_a (rows x cols);  else psi_a (rows x cols) rot_b^T (cols x im)
        uint64_t wpos = 0;
        std::vector<uint64_t> out_off(na, 0), out_sz(na, 0);
        for (int a = 0; a < na; a++) {
            const int b = lay->psi_dm[a];
            if (b < 0 || kept[b] == 0)
                continue;
            const int r = lay->psi_rows[a], c = lay->psi_cols[a], im = kept[b];
            out_off[a] = wpos;
            if ((uint64_t)r * c == 0)
                continue;
            if (tr) {
                out_sz[a] = (uint64_t)im * c;
                small_gemm<<<(unsigned)((out_sz[a] + 255) / 256), 256, 0, s>>>(
                    d_out + wpos, d_rot + rot_off[b], im, 1, d_psi + lay->psi_off[a], c, 0, im, c, r);
            } else {
                out_sz[a] = (uint64_t)r * im;
                small_gemm<<<(unsigned)((out_sz[a] + 255) / 256), 256, 0, s>>>(
                    d_out + wpos, d_psi + lay->psi_off[a], c, 0, d_rot + rot_off[b], lay->dm_dim[b], 1, r, im, c);
            }
            DM_TRY(cudaGetLastError());
            wpos += out_sz[a];
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
