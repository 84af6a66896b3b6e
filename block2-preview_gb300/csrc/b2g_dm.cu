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
// per block, parallel cyclic Jacobi with round-robin pairing, matrix and
// eigenvectors in global memory so blocks of any size fit), and the split
// GEMMs.  The selection of the kept states (a sort of at most a few thousand
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

// One CTA per block: cyclic Jacobi, round-robin pairs (index 0 fixed).
// A (n x n, symmetric, destroyed) -> eigenvalues w (ascending), eigenvectors
// as ROWS of V (row j = eigenvector of w[j], the storage LAPACK leaves in a
// row-major matrix).  Vt holds the accumulated rotation (columns = vectors).
constexpr int kJacThreads = 256;
constexpr int kJacMaxHalf = 1024;  // blocks up to 2048 states
constexpr int kJacMaxSweeps = 60;
__global__ void __launch_bounds__(kJacThreads) jacobi_block(double *__restrict__ Aall,
                                                            double *__restrict__ Vtall,
                                                            double *__restrict__ Vall,
                                                            const int32_t *__restrict__ dim,
                                                            const uint64_t *__restrict__ off,
                                                            double *__restrict__ wall,
                                                            const uint64_t *__restrict__ woff,
                                                            int *__restrict__ perm_all,
                                                            int *err) {
    __shared__ double cs[kJacMaxHalf], sn[kJacMaxHalf];
    __shared__ int pp[kJacMaxHalf], qq[kJacMaxHalf];
    __shared__ double red[kJacThreads / 32];
    __shared__ double thr_s;
    __shared__ int rotated_s;
    const int b = blockIdx.x;
    const int n = dim[b];
    if (n == 0)
        return;
    double *A = Aall + off[b], *Vt = Vtall + off[b], *V = Vall + off[b], *w = wall + woff[b];
    int *perm = perm_all + woff[b] + b;  // n + 1 slots per block
    const int tid = threadIdx.x;
    const int mm = n + (n & 1), half = mm / 2;
    if (half > kJacMaxHalf) {
        if (tid == 0)
            atomicExch(err, 1);
        return;
    }
    for (int64_t e = tid; e < (int64_t)n * n; e += kJacThreads)
        Vt[e] = (e / n == e % n) ? 1.0 : 0.0;
    for (int i = tid; i < mm; i += kJacThreads)
        perm[i] = i;
    __syncthreads();
    // rotation threshold: 1e-18 of the Frobenius norm, far below the
    // eps * |A| absolute accuracy LAPACK's dsyev gives
    {
        double st = 0.0;
        for (int64_t e = tid; e < (int64_t)n * n; e += kJacThreads)
            st += A[e] * A[e];
        for (int o = 16; o > 0; o >>= 1)
            st += __shfl_down_sync(0xffffffffu, st, o);
        if ((tid & 31) == 0)
            red[tid >> 5] = st;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int k = 0; k < kJacThreads / 32; k++)
                t += red[k];
            thr_s = 1e-18 * sqrt(t);
        }
        __syncthreads();
    }
    const double thr = thr_s;
    for (int sweep = 0; sweep < kJacMaxSweeps; sweep++) {
        if (tid == 0)
            rotated_s = 0;
        __syncthreads();
        for (int step = 0; step < mm - 1; step++) {
            for (int k = tid; k < half; k += kJacThreads) {
                int p = perm[k], q = perm[mm - 1 - k];
                if (p > q) {
                    const int t = p;
                    p = q, q = t;
                }
                pp[k] = p, qq[k] = q;
                double c = 1.0, s = 0.0;
                if (q < n) {
                    const double apq = A[(int64_t)p * n + q];
                    if (fabs(apq) > thr) {
                        rotated_s = 1;
                        const double th = (A[(int64_t)q * n + q] - A[(int64_t)p * n + p]) / (2.0 * apq);
                        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                        c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                    }
                }
                cs[k] = c, sn[k] = s;
            }
            __syncthreads();
            // columns: A <- A J, Vt <- Vt J
            for (int64_t e = tid; e < (int64_t)half * n; e += kJacThreads) {
                const int k = (int)(e / n), r = (int)(e % n), p = pp[k], q = qq[k];
                if (q >= n || sn[k] == 0.0)
                    continue;
                const double c = cs[k], s = sn[k];
                double *Ar = A + (int64_t)r * n, *Vr = Vt + (int64_t)r * n;
                const double arp = Ar[p], arq = Ar[q];
                Ar[p] = c * arp - s * arq, Ar[q] = s * arp + c * arq;
                const double vrp = Vr[p], vrq = Vr[q];
                Vr[p] = c * vrp - s * vrq, Vr[q] = s * vrp + c * vrq;
            }
            __syncthreads();
            // rows: A <- J^T A
            for (int64_t e = tid; e < (int64_t)half * n; e += kJacThreads) {
                const int k = (int)(e / n), cidx = (int)(e % n), p = pp[k], q = qq[k];
                if (q >= n || sn[k] == 0.0)
                    continue;
                const double c = cs[k], s = sn[k];
                const double apc = A[(int64_t)p * n + cidx], aqc = A[(int64_t)q * n + cidx];
                // the eliminated pair is set to zero exactly
                A[(int64_t)p * n + cidx] = cidx == q ? 0.0 : c * apc - s * aqc;
                A[(int64_t)q * n + cidx] = cidx == p ? 0.0 : s * apc + c * aqc;
            }
            __syncthreads();
            if (tid == 0) {
                const int last = perm[mm - 1];
                for (int k = mm - 1; k > 1; k--)
                    perm[k] = perm[k - 1];
                perm[1] = last;
            }
            __syncthreads();
        }
        if (rotated_s == 0)
            break;
        __syncthreads();
    }
    // sort ascending (selection sort by one thread; n is at most a few hundred)
    if (tid == 0) {
        for (int i = 0; i < n; i++)
            perm[i] = i;
        for (int i = 0; i < n; i++) {
            int bi = i;
            for (int j = i + 1; j < n; j++)
                if (A[(int64_t)perm[j] * n + perm[j]] < A[(int64_t)perm[bi] * n + perm[bi]])
                    bi = j;
            const int t = perm[i];
            perm[i] = perm[bi], perm[bi] = t;
        }
        for (int i = 0; i < n; i++)
            w[i] = A[(int64_t)perm[i] * n + perm[i]];
    }
    __syncthreads();
    for (int64_t e = tid; e < (int64_t)n * n; e += kJacThreads) {
        const int j = (int)(e / n), r = (int)(e % n);  // V row j = column perm[j] of Vt
        V[e] = Vt[(int64_t)r * n + perm[j]];
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
            jacobi_block<<<nb, kJacThreads, 0, s>>>(d_rho, d_vt, d_v, d_dim, d_roff, d_w, d_woff, d_perm, d_err);
            DM_TRY(cudaGetLastError());
        }
        std::vector<double> w(wtot);
        int errflag = 0;
        DM_TRY(cudaMemcpyAsync(w.data(), d_w, sizeof(double) * wtot, cudaMemcpyDeviceToHost, s));
        DM_TRY(cudaMemcpyAsync(&errflag, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        DM_TRY(cudaStreamSynchronize(s));
        if (errflag) {
            rc = fail(B2G_ERR_UNSUPPORTED, "b2g_dm_truncate: density-matrix block above 2048 states");
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
