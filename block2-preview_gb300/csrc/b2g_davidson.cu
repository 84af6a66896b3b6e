// Device-resident Davidson eigensolver for the lowest eigenpair(s) of H_eff.
//
// Restates IterativeMatrixFunctions::davidson, Normal type, Olsen
// preconditioner (src/core/iterative_matrix_functions.hpp:864-1173, 93-108)
// with the same basis growth, convergence test (|r|^2 < conv_thrd), restart
// to def_min vectors when def_max is reached, and orthogonalisation of the
// correction vectors.  One root (b2g_davidson) or k state-averaged roots
// (b2g_davidson_multi): the block variant adds the corrections of all
// unconverged roots per iteration and applies H_eff to them in one
// b2g_heff_apply_batch call.  In a reduced-precision form (FP32, TF32x3) the
// products are reduced-precision and convergence is only declared on an FP64
// residual of the Ritz vector (defect correction; the energy returned is the
// FP64 Rayleigh quotient).  Arithmetic differences from the reference, all
// exact in exact arithmetic:
//   * the basis is not rotated to Ritz vectors every iteration; the Ritz
//     vector x = B v and its H-image s = Sigma v are formed directly and the
//     subspace matrix grows by one row per new vector (the reference rotates
//     all m vectors and recomputes all m^2 dot products each iteration);
//     the rotation to the def_min lowest Ritz vectors happens only at restart;
//   * the small subspace eigenproblem (LAPACK dsyev in the reference) is
//     solved on the device by threshold cyclic Jacobi (one CTA, FP64),
//     warm-started from the previous iteration's eigenvectors;
//   * the correction vector is orthogonalised by classical Gram-Schmidt
//     applied twice (the reference applies modified Gram-Schmidt once).
// All vectors live in HBM; per iteration only the Ritz values and residual
// norms come back to the host for the convergence decision.  Reductions are two-stage
// (per-block partials, then a fixed-order sum): results are bit-reproducible.
#include <algorithm>
#include <cmath>
#include <vector>

#include "b2g_internal.h"

namespace b2g {

namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 304;   // 2 x 152 SMs
constexpr int kMaxSub = 64;       // def_max limit (Jacobi in one CTA)

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// out[j] = X_j . y for j < nv (X_j = X + j * ldx), one launch: every block
// sums its grid-stride slice for up to kDotBatch vectors at a time (independent
// FP64 chains, interleaved reductions) into partial[j * gridDim.x + block];
// the last block to finish (a counter, reset by that block) adds the
// partials of each j in block order.  Deterministic: fixed slices, fixed
// reduction trees, fixed final order.
constexpr int kDotBatch = 8;
// NB vectors j0 .. j0+NB-1 of this block's slice into partial; exact NB so the
// narrow FP64 pipe issues no predicated-off FMA or add
template <int NB>
__device__ __forceinline__ void multidot_chunk(const double *__restrict__ X, uint64_t ldx, int j0,
                                               const double *__restrict__ y, uint64_t n,
                                               double *partial, double (*red)[kDotBatch]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    double s[NB];
#pragma unroll
    for (int jj = 0; jj < NB; jj++)
        s[jj] = 0.0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double yi = y[i];
#pragma unroll
        for (int jj = 0; jj < NB; jj++)
            s[jj] = fma(X[(uint64_t)(j0 + jj) * ldx + i], yi, s[jj]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int jj = 0; jj < NB; jj++)
            s[jj] += __shfl_down_sync(0xffffffffu, s[jj], o);
    if (lane == 0)
#pragma unroll
        for (int jj = 0; jj < NB; jj++)
            red[warp][jj] = s[jj];
    __syncthreads();
    if (threadIdx.x < NB) {
        const int jj = threadIdx.x;
        static_assert(kRedThreads / 32 == 8, "tree below sums 8 warps");
        const double v = ((red[0][jj] + red[1][jj]) + (red[2][jj] + red[3][jj])) +
                         ((red[4][jj] + red[5][jj]) + (red[6][jj] + red[7][jj]));
        partial[(uint64_t)(j0 + jj) * gridDim.x + blockIdx.x] = v;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kRedThreads) multidot(const double *__restrict__ X, uint64_t ldx,
                                                        int nv, const double *__restrict__ y,
                                                        uint64_t n, double *partial,
                                                        unsigned *counter, double *out) {
    __shared__ double red[kRedThreads / 32][kDotBatch];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j0 = 0; j0 < nv; j0 += kDotBatch) {
        switch (min(kDotBatch, nv - j0)) {
        case 1: multidot_chunk<1>(X, ldx, j0, y, n, partial, red); break;
        case 2: multidot_chunk<2>(X, ldx, j0, y, n, partial, red); break;
        case 3: multidot_chunk<3>(X, ldx, j0, y, n, partial, red); break;
        case 4: multidot_chunk<4>(X, ldx, j0, y, n, partial, red); break;
        case 5: multidot_chunk<5>(X, ldx, j0, y, n, partial, red); break;
        case 6: multidot_chunk<6>(X, ldx, j0, y, n, partial, red); break;
        case 7: multidot_chunk<7>(X, ldx, j0, y, n, partial, red); break;
        default: multidot_chunk<8>(X, ldx, j0, y, n, partial, red); break;
        }
    }
    // the last block adds the partials
    __threadfence();
    if (threadIdx.x == 0)
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last)
        return;
    __threadfence();
    for (int j = warp; j < nv; j += kRedThreads / 32) {
        double v = 0.0;
        for (int bb = lane; bb < (int)gridDim.x; bb += 32)
            v += __ldcg(partial + (uint64_t)j * gridDim.x + bb);
        v = warp_sum(v);
        if (lane == 0)
            out[j] = v;
    }
    if (threadIdx.x == 0)
        *counter = 0u;
}

// y = beta * y + sum_j coef[j] * X_j   (coef on device, optionally negated)
__global__ void combine(double *__restrict__ y, double beta, const double *__restrict__ X,
                        uint64_t ldx, int nv, const double *__restrict__ coef, double coef_sign,
                        uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double s = beta == 0.0 ? 0.0 : beta * y[i];
        for (int j = 0; j < nv; j++)
            s = fma(coef_sign * coef[j], X[(uint64_t)j * ldx + i], s);
        y[i] = s;
    }
}

// Y_j = sum_i X_i V[i, j] for j < nout (V row-major ldv) -- restart rotation
__global__ void rotate_basis(double *__restrict__ Y, const double *__restrict__ X, uint64_t ld,
                             int m, int nout, const double *__restrict__ V, int ldv, uint64_t n) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        for (int j = 0; j < nout; j++) {
            double s = 0.0;
            for (int k = 0; k < m; k++)
                s = fma(X[(uint64_t)k * ld + i], V[k * ldv + j], s);
            Y[(uint64_t)j * ld + i] = s;
        }
}

// q = s - lambda x ; in the same pass the Olsen quantities
//   t = x / (lambda - d), q' = q / (lambda - d) where |lambda - d| > 1e-12
__global__ void residual_olsen(double *__restrict__ q, double *__restrict__ t,
                               const double *__restrict__ s, const double *__restrict__ x,
                               const double *__restrict__ diag, const double *__restrict__ lam,
                               uint64_t n, int precondition) {
    const double l = lam[0];
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        double qi = s[i] - l * x[i];
        double ti = x[i];
        if (precondition) {
            const double den = l - diag[i];
            if (fabs(den) > 1e-12)
                qi /= den, ti /= den;
        }
        q[i] = qi;
        t[i] = ti;
    }
}

// q -= (d[0] / d[1]) * t   (Olsen: (x, K^-1 q) / (x, K^-1 x))
__global__ void olsen_update(double *__restrict__ q, const double *__restrict__ t,
                             const double *__restrict__ d, uint64_t n) {
    const double r = d[0] / d[1];
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        q[i] = fma(-r, t[i], q[i]);
}

// y = x / sqrt(d[0])
__global__ void normalize_into(double *__restrict__ y, const double *__restrict__ x,
                               const double *__restrict__ d, uint64_t n) {
    // a (numerically) zero vector becomes zero: the host drops it afterwards
    const double f = d[0] > 1e-28 ? 1.0 / sqrt(d[0]) : 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        y[i] = x[i] * f;
}

// Parallel cyclic Jacobi on the m x m symmetric matrix A (row-major, lda), one
// CTA.  Outputs eigenvalues ascending in w[0..m) and eigenvectors as columns
// of V (row-major, ldv = kMaxSub).  Round s of a sweep pairs the indices by
// the circle method (0 with 1 + s, and 1 + (s + j) with 1 + (s - j) modulo
// mm - 1), so every pair meets once per sweep.  Rotations whose off-diagonal
// element is below 1e-17 of the Frobenius norm are skipped (threshold
// Jacobi): the FP64 pipe of one SM is the limit here, and a warm-started or
// late sweep touches few pairs.  Stops when the off-diagonal mass is below
// 1e-30 of the total or a sweep rotates nothing.
__global__ void __launch_bounds__(256) jacobi_eig(const double *__restrict__ Ain, int lda, int m,
                                                  double *__restrict__ w, double *__restrict__ V) {
    __shared__ double A[kMaxSub][kMaxSub + 1];
    __shared__ double Vs[kMaxSub][kMaxSub + 1];
    __shared__ double cs[kMaxSub / 2], sn[kMaxSub / 2];
    __shared__ int pp[kMaxSub / 2], qq[kMaxSub / 2];
    __shared__ int n_act, n_rot, perm[kMaxSub];
    __shared__ double red_off[8], red_tot[8], thr_s, stop_s;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
    const int mm = m + (m & 1);  // padded to even: the extra index is a dummy
    for (int i = tid; i < mm * mm; i += nt) {
        const int r = i / mm, c = i % mm;
        A[r][c] = (r < m && c < m) ? Ain[r * lda + c] : 0.0;
        Vs[r][c] = r == c ? 1.0 : 0.0;
    }
    __syncthreads();
    const int half = mm / 2, n1 = mm - 1;
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = tid; i < m * m; i += nt) {
            const int r = i / m, c = i % m;
            const double v = A[r][c] * A[r][c];
            (r == c ? tot : off) += v;
        }
        off = warp_sum(off), tot = warp_sum(tot);
        if (lane == 0)
            red_off[wid] = off, red_tot[wid] = tot;
        __syncthreads();
        if (tid == 0) {
            double o = 0.0, t = 0.0;
            for (int i = 0; i < nt / 32; i++)
                o += red_off[i], t += red_tot[i];
            stop_s = (o <= 1e-30 * (t + o)) ? 1.0 : 0.0;
            thr_s = 1e-17 * sqrt(t + o);
            n_rot = 0;
        }
        __syncthreads();
        if (stop_s != 0.0)
            break;
        const double thr = thr_s;
        for (int step = 0; step < n1; step++) {
            if (tid == 0)
                n_act = 0;
            __syncthreads();
            for (int k = tid; k < half; k += nt) {
                int p = k == 0 ? 0 : 1 + (step + k) % n1;
                int q = 1 + (step + n1 - k) % n1;
                if (k == 0)
                    q = 1 + step % n1;
                if (p > q) {
                    const int t = p;
                    p = q, q = t;
                }
                if (q < m && fabs(A[p][q]) > thr) {
                    const double th = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                    const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                    const double c = 1.0 / sqrt(t * t + 1.0);
                    const int slot = atomicAdd(&n_act, 1);  // pairs are disjoint: order is immaterial
                    pp[slot] = p, qq[slot] = q, cs[slot] = c, sn[slot] = t * c;
                }
            }
            __syncthreads();
            const int na = n_act;
            if (na == 0)
                continue;  // uniform: every thread read the same count
            if (tid == 0)
                n_rot += na;
            // columns: A <- A J, V <- V J
            for (int i = tid; i < na * mm; i += nt) {
                const int k = i / mm, r = i % mm, p = pp[k], q = qq[k];
                const double c = cs[k], s = sn[k];
                const double arp = A[r][p], arq = A[r][q];
                A[r][p] = c * arp - s * arq;
                A[r][q] = s * arp + c * arq;
                const double vrp = Vs[r][p], vrq = Vs[r][q];
                Vs[r][p] = c * vrp - s * vrq;
                Vs[r][q] = s * vrp + c * vrq;
            }
            __syncthreads();
            // rows: A <- J^T A
            for (int i = tid; i < na * mm; i += nt) {
                const int k = i / mm, r = i % mm, p = pp[k], q = qq[k];
                const double c = cs[k], s = sn[k];
                const double apr = A[p][r], aqr = A[q][r];
                A[p][r] = c * apr - s * aqr;
                A[q][r] = s * apr + c * aqr;
            }
            __syncthreads();
        }
        __syncthreads();
        if (n_rot == 0)
            break;
    }
    if (tid == 0) {
        // sort ascending (selection), record order in perm
        for (int i = 0; i < m; i++)
            perm[i] = i;
        for (int i = 0; i < m; i++) {
            int b = i;
            for (int j = i + 1; j < m; j++)
                if (A[perm[j]][perm[j]] < A[perm[b]][perm[b]])
                    b = j;
            const int t = perm[i];
            perm[i] = perm[b], perm[b] = t;
        }
        for (int i = 0; i < m; i++)
            w[i] = A[perm[i]][perm[i]];
    }
    __syncthreads();
    for (int i = tid; i < m * m; i += nt) {
        const int r = i / m, c = i % m;
        V[r * kMaxSub + c] = Vs[r][perm[c]];
    }
}

// Warm start of the subspace eigenproblem: with the previous eigenvectors
// Vp (mw x mw, ld kMaxSub) of the leading block, which the new basis vectors
// only border, E = blockdiag(Vp, I) turns A into E^T A E, diagonal but for the
// new rows, so Jacobi touches few pairs; the eigenvectors are then E times
// Jacobi's.  One CTA per row (these products are O(m^3) FP64 work, spread
// over m SMs).
// T = A E
__global__ void __launch_bounds__(64) sub_warm_right(const double *__restrict__ A, int m, int mw,
                                                     const double *__restrict__ Vp,
                                                     double *__restrict__ T) {
    const int r = blockIdx.x;
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        double v = 0.0;
        if (c < mw) {
            for (int b = 0; b < mw; b++)
                v = fma(A[r * kMaxSub + b], Vp[b * kMaxSub + c], v);
        } else {
            v = A[r * kMaxSub + c];
        }
        T[r * kMaxSub + c] = v;
    }
}
// A2 = E^T T
__global__ void __launch_bounds__(64) sub_warm_left(const double *__restrict__ T, int m, int mw,
                                                    const double *__restrict__ Vp,
                                                    double *__restrict__ A2) {
    const int r = blockIdx.x;
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        double v = 0.0;
        if (r < mw) {
            for (int a = 0; a < mw; a++)
                v = fma(Vp[a * kMaxSub + r], T[a * kMaxSub + c], v);
        } else {
            v = T[r * kMaxSub + c];
        }
        A2[r * kMaxSub + c] = v;
    }
}
// V = E Vj
__global__ void __launch_bounds__(64) sub_warm_vec(const double *__restrict__ Vp, int m, int mw,
                                                   const double *__restrict__ Vj,
                                                   double *__restrict__ V) {
    const int r = blockIdx.x;
    for (int c = threadIdx.x; c < m; c += blockDim.x) {
        double v = 0.0;
        if (r < mw) {
            for (int b = 0; b < mw; b++)
                v = fma(Vp[r * kMaxSub + b], Vj[b * kMaxSub + c], v);
        } else {
            v = Vj[r * kMaxSub + c];
        }
        V[r * kMaxSub + c] = v;
    }
}

// A[i * lda + j] = A[j * lda + i] = v[j] for j <= i (new subspace row)
__global__ void set_sub_row(double *A, int lda, int i, const double *v) {
    const int j = threadIdx.x;
    if (j <= i) {
        A[i * lda + j] = v[j];
        A[j * lda + i] = v[j];
    }
}

// A = diag(w[0..m)) (restart)
__global__ void set_sub_diag(double *A, int lda, int m, const double *w) {
    for (int i = threadIdx.x; i < lda * lda; i += blockDim.x) {
        const int r = i / lda, c = i % lda;
        A[i] = (r == c && r < m) ? w[r] : 0.0;
    }
}

int grid_for(uint64_t n) {
    uint64_t b = (n + 255) / 256;
    return (int)std::min<uint64_t>(b ? b : 1, 152 * 8);
}

} // namespace

} // namespace b2g

using namespace b2g;

// Block Davidson for the k lowest eigenpairs.  k = 1 is the reference's
// one-root Davidson; for k > 1 every unconverged root contributes its Olsen
// correction each iteration and all new basis vectors go through one batched
// H_eff product (the reference converges state-averaged roots one correction
// at a time, iterative_matrix_functions.hpp:1010-1160; the converged
// eigenpairs are the same).
static int davidson_impl(b2g_heff *h, const double *diag, double *psi, int k, double conv_thrd,
                         int max_iter, int def_min, int def_max, int form, double *energies,
                         b2g_davidson_result *res) {
    if (h == nullptr || diag == nullptr || psi == nullptr || res == nullptr || k < 1)
        return fail(B2G_ERR_ARG, "b2g_davidson: null argument or k < 1");
    if (h->psi_size != h->sigma_size)
        return fail(B2G_ERR_ARG, "b2g_davidson: H_eff is not square (bra != ket size)");
    if (form != B2G_FP64 && form != B2G_FP32 && form != B2G_TF32X3)
        return fail(B2G_ERR_UNSUPPORTED, "b2g_davidson: unknown form");
    def_min = std::max(def_min, k);
    def_max = std::max(def_max, def_min + k);
    if (def_max > kMaxSub)
        return fail(B2G_ERR_ARG, "b2g_davidson: def_max above 64");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    cudaStream_t st = h->ctx->stream;
    const uint64_t n = h->psi_size;
    const int g = grid_for(n);
    double *B = nullptr, *S = nullptr, *X = nullptr, *SX = nullptr, *Q = nullptr, *t = nullptr,
           *R = nullptr, *D = nullptr, *small = nullptr, *partial = nullptr;
    const size_t nsmall = (size_t)kMaxSub * kMaxSub * 6 + 6 * kMaxSub + 16;
    auto cleanup = [&]() {
        cudaFree(B), cudaFree(S), cudaFree(X), cudaFree(SX), cudaFree(Q), cudaFree(t), cudaFree(R);
        cudaFree(D), cudaFree(small), cudaFree(partial);
    };
    if (cudaMalloc(&B, sizeof(double) * n * def_max) || cudaMalloc(&S, sizeof(double) * n * def_max) ||
        cudaMalloc(&X, sizeof(double) * n * k) || cudaMalloc(&SX, sizeof(double) * n * k) ||
        cudaMalloc(&Q, sizeof(double) * n * k) || cudaMalloc(&t, sizeof(double) * n) ||
        cudaMalloc(&R, sizeof(double) * n * def_min) || cudaMalloc(&D, sizeof(double) * n) ||
        cudaMalloc(&small, sizeof(double) * nsmall) ||
        cudaMalloc(&partial, sizeof(double) * (kRedBlocks * kMaxSub + 1))) {
        cleanup();
        return fail(B2G_ERR_NOMEM, "b2g_davidson: device workspace allocation failed");
    }
    double *A = small;                          // kMaxSub x kMaxSub subspace matrix
    double *V = A + kMaxSub * kMaxSub;          // eigenvectors (columns), ld kMaxSub
    double *Vprev = V + kMaxSub * kMaxSub;      // the previous Ritz solve's eigenvectors
    double *T = Vprev + kMaxSub * kMaxSub;      // warm-start scratch (A E, then Jacobi's vectors)
    double *A2 = T + kMaxSub * kMaxSub;         // E^T A E
    double *w = A2 + 2 * kMaxSub * kMaxSub;     // eigenvalues (ascending)
    double *dots = w + kMaxSub;                 // kMaxSub dot results
    double *qqd = dots + kMaxSub;               // kMaxSub residual norms
    double *sc = qqd + kMaxSub;                 // scratch scalars
    double *coef = sc + 16;                     // kMaxSub coefficients
    unsigned *dot_counter = (unsigned *)(partial + (size_t)kRedBlocks * kMaxSub);
    // about four elements per thread: short per-thread FP64 chains and few partials
    const int dot_blocks = (int)std::min<uint64_t>(kRedBlocks, std::max<uint64_t>(1, (n + 1023) / 1024));
    auto dot_many = [&](const double *Xv, int nv, const double *y, double *out) {
        note_launch();
        multidot<<<dot_blocks, kRedThreads, 0, st>>>(Xv, n, nv, y, n, partial, dot_counter, out);
    };
    std::vector<double> lam(kMaxSub), qq(kMaxSub);
    int rc = B2G_OK;
    int m = 0, msig = 0, xiter = 0, n_fp64 = 0, n_mixed = 0, n_refine = 0, since_refine = 0;
    int vw = 0;  // leading block of A whose eigenvectors V holds (warm start), 0 = none
    bool converged = false, have_exact = false;
    // host-side helpers; each returns false after recording an error in rc
    auto cuda_ok = [&](cudaError_t e, const char *what) {
        if (e == cudaSuccess)
            return true;
        rc = fail(B2G_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
        return false;
    };
    // orthogonalise Q_row (device vector q) against B[0..m) twice, append if not degenerate
    auto append = [&](double *q) -> int {
        for (int pass = 0; pass < 2 && m > 0; pass++) {
            dot_many(B, m, q, coef);
            note_launch();
            combine<<<g, 256, 0, st>>>(q, 1.0, B, n, m, coef, -1.0, n);
        }
        dot_many(q, 1, q, sc + 1);
        double nrm2 = 0;
        if (!cuda_ok(cudaMemcpyAsync(&nrm2, sc + 1, sizeof(double), cudaMemcpyDeviceToHost, st), "norm") ||
            !cuda_ok(cudaStreamSynchronize(st), "sync"))
            return -1;
        if (!(nrm2 > 1e-28))
            return 0;
        note_launch();
        normalize_into<<<g, 256, 0, st>>>(B + (uint64_t)m * n, q, sc + 1, n);
        m++;
        return 1;
    };
    // sigma of the new basis vectors [msig, m) in one batched product, subspace rows
    auto expand = [&](int pform) -> bool {
        const int nn = m - msig;
        if (nn <= 0)
            return true;
        if (!cuda_ok(cudaMemsetAsync(S + (uint64_t)msig * n, 0, sizeof(double) * n * nn, st), "memset"))
            return false;
        rc = b2g_heff_apply_batch(h, B + (uint64_t)msig * n, S + (uint64_t)msig * n, nn, 1.0, pform);
        if (rc != B2G_OK)
            return false;
        (pform == B2G_FP64 ? n_fp64 : n_mixed) += nn;
        for (int i = msig; i < m; i++) {
            dot_many(S, i + 1, B + (uint64_t)i * n, dots);
            note_launch();
            set_sub_row<<<1, kMaxSub, 0, st>>>(A, kMaxSub, i, dots);
        }
        msig = m;
        return true;
    };
    // Rayleigh-Ritz: X, SX = the k lowest Ritz vectors and their images, residual norms
    auto ritz = [&]() -> bool {
        if (vw > 0 && vw < m) {
            std::swap(V, Vprev);
            note_launch();
            sub_warm_right<<<m, 64, 0, st>>>(A, m, vw, Vprev, T);
            note_launch();
            sub_warm_left<<<m, 64, 0, st>>>(T, m, vw, Vprev, A2);
            note_launch();
            jacobi_eig<<<1, 256, 0, st>>>(A2, kMaxSub, m, w, T);
            note_launch();
            sub_warm_vec<<<m, 64, 0, st>>>(Vprev, m, vw, T, V);
        } else {
            note_launch();
            jacobi_eig<<<1, 256, 0, st>>>(A, kMaxSub, m, w, V);
        }
        vw = m;
        note_launch();
        rotate_basis<<<g, 256, 0, st>>>(X, B, n, m, k, V, kMaxSub, n);
        note_launch();
        rotate_basis<<<g, 256, 0, st>>>(SX, S, n, m, k, V, kMaxSub, n);
        for (int i = 0; i < k; i++) {
            note_launch();
            residual_olsen<<<g, 256, 0, st>>>(Q + (uint64_t)i * n, t, SX + (uint64_t)i * n,
                                              X + (uint64_t)i * n, D, w + i, n, 0);
            dot_many(Q + (uint64_t)i * n, 1, Q + (uint64_t)i * n, qqd + i);
        }
        return cuda_ok(cudaMemcpyAsync(lam.data(), w, sizeof(double) * m, cudaMemcpyDeviceToHost, st), "w") &&
               cuda_ok(cudaMemcpyAsync(qq.data(), qqd, sizeof(double) * k, cudaMemcpyDeviceToHost, st), "qq") &&
               cuda_ok(cudaStreamSynchronize(st), "sync");
    };
    // Threshold on the residual the reduced-precision products estimate, per
    // root.  Before any FP64 product: 1e-10 lam^2, safely above the noise floor
    // of a reduced product of an eigenvalue of size lam (a TF32x3 product is
    // good to a few 1e-6 relative), so the reduced Davidson has settled on the
    // lowest states before the first FP64 product collapses the basis onto its
    // Ritz vectors.  After an FP64 certification that left exact residuals
    // qq_exact: four orders of magnitude below the largest of them (each
    // reduced cycle has to earn its next FP64 product).  Never below conv_thrd;
    // the FP64 form uses conv_thrd throughout.
    double qq_exact = 0.0;
    auto red_thr = [&](bool reduced, int i) {
        if (!reduced)
            return conv_thrd;
        if (!have_exact)
            return std::max(conv_thrd, 1e-10 * lam[i] * lam[i]);
        return std::max(conv_thrd, 1e-4 * qq_exact);
    };
    auto all_below = [&](bool reduced) {
        for (int i = 0; i < k; i++)
            if (!(qq[i] < red_thr(reduced, i)))
                return false;
        return true;
    };
    auto all_below_exact = [&]() {
        for (int i = 0; i < k; i++)
            if (!(qq[i] < conv_thrd))
                return false;
        return true;
    };
    // ---- initial basis: the k guesses, orthonormalised
    if (!cuda_ok(cudaMemcpyAsync(D, diag, sizeof(double) * n, cudaMemcpyHostToDevice, st), "diag") ||
        !cuda_ok(cudaMemcpyAsync(Q, psi, sizeof(double) * n * k, cudaMemcpyHostToDevice, st), "psi") ||
        !cuda_ok(cudaMemsetAsync(A, 0, sizeof(double) * kMaxSub * kMaxSub, st), "A") ||
        !cuda_ok(cudaMemsetAsync(dot_counter, 0, sizeof(unsigned), st), "counter"))
        goto done;
    for (int i = 0; i < k; i++) {
        const int r = append(Q + (uint64_t)i * n);
        if (r < 0)
            goto done;
        if (r == 0) {
            rc = fail(B2G_ERR_ARG, "b2g_davidson: initial guesses are linearly dependent");
            goto done;
        }
    }
    while (xiter < max_iter) {
        xiter++;
        since_refine++;
        if (!expand(form) || !ritz())
            goto done;
        const bool reduced = form != B2G_FP64;
        // reduced cycles are also cut off after a fixed number of iterations
        // (longer before the first FP64 product, while the lowest states are
        // still being found)
        if (all_below(reduced) || (reduced && since_refine >= (have_exact ? 40 : 200))) {
            if (!reduced) {
                converged = true;
                break;
            }
            // Defect correction: FP64 products of the k Ritz vectors; Rayleigh-Ritz
            // in their span with exact sigmas; converged when every exact residual
            // is below conv_thrd, otherwise continue from this exact basis.
            if (!cuda_ok(cudaMemcpyAsync(B, X, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st), "X"))
                goto done;
            m = k, msig = 0, vw = 0;
            if (!cuda_ok(cudaMemsetAsync(A, 0, sizeof(double) * kMaxSub * kMaxSub, st), "A") ||
                !expand(B2G_FP64) || !ritz())
                goto done;
            if (all_below_exact()) {
                converged = true;
                break;
            }
            if (++n_refine > 30)
                break;
            have_exact = true;
            qq_exact = *std::max_element(qq.begin(), qq.begin() + k);
            since_refine = 0;
        }
        // ---- restart when the new corrections would not fit
        int n_unconv = 0;
        for (int i = 0; i < k; i++)
            n_unconv += qq[i] >= red_thr(reduced, i);
        if (m + n_unconv > def_max) {
            note_launch();
            rotate_basis<<<g, 256, 0, st>>>(R, B, n, m, def_min, V, kMaxSub, n);
            if (!cuda_ok(cudaMemcpyAsync(B, R, sizeof(double) * n * def_min, cudaMemcpyDeviceToDevice, st), "B"))
                goto done;
            note_launch();
            rotate_basis<<<g, 256, 0, st>>>(R, S, n, m, def_min, V, kMaxSub, n);
            if (!cuda_ok(cudaMemcpyAsync(S, R, sizeof(double) * n * def_min, cudaMemcpyDeviceToDevice, st), "S"))
                goto done;
            note_launch();
            set_sub_diag<<<1, 256, 0, st>>>(A, kMaxSub, def_min, w);
            m = msig = def_min;
            vw = 0;
        }
        // ---- Olsen corrections of the unconverged roots, appended in order
        // (Gram-Schmidt twice against the basis including the corrections
        // appended before them) without a host round trip per root: each norm
        // lands in dots[], a numerically zero correction is stored as a zero
        // vector, and one read of the norms afterwards drops those
        int added = 0, mp = m;
        for (int i = 0; i < k; i++) {
            if (qq[i] < red_thr(reduced, i) || mp >= def_max)
                continue;
            double *q = Q + (uint64_t)i * n, *x = X + (uint64_t)i * n;
            note_launch();
            residual_olsen<<<g, 256, 0, st>>>(q, t, SX + (uint64_t)i * n, x, D, w + i, n, 1);
            dot_many(q, 1, x, sc + 2);
            dot_many(t, 1, x, sc + 3);
            note_launch();
            olsen_update<<<g, 256, 0, st>>>(q, t, sc + 2, n);
            for (int pass = 0; pass < 2 && mp > 0; pass++) {
                dot_many(B, mp, q, coef);
                note_launch();
                combine<<<g, 256, 0, st>>>(q, 1.0, B, n, mp, coef, -1.0, n);
            }
            dot_many(q, 1, q, dots + (mp - m));
            note_launch();
            normalize_into<<<g, 256, 0, st>>>(B + (uint64_t)mp * n, q, dots + (mp - m), n);
            mp++;
        }
        if (mp > m) {
            std::vector<double> nr(mp - m);
            if (!cuda_ok(cudaMemcpyAsync(nr.data(), dots, sizeof(double) * (mp - m), cudaMemcpyDeviceToHost, st),
                         "norms") ||
                !cuda_ok(cudaStreamSynchronize(st), "sync"))
                goto done;
            for (int j = 0; j < mp - m; j++) {
                if (!(nr[j] > 1e-28))
                    continue;  // dropped (stored as zeros, never used)
                if (m + added != m + j &&
                    !cuda_ok(cudaMemcpyAsync(B + (uint64_t)(m + added) * n, B + (uint64_t)(m + j) * n,
                                             sizeof(double) * n, cudaMemcpyDeviceToDevice, st), "compact"))
                    goto done;
                added++;
            }
            m += added;
        }
        if (added == 0 && msig == m)
            break;  // no new direction: stagnated
    }
    if (!cuda_ok(cudaGetLastError(), "kernels") ||
        !cuda_ok(cudaMemcpyAsync(psi, X, sizeof(double) * n * k, cudaMemcpyDeviceToHost, st), "psi out") ||
        !cuda_ok(cudaStreamSynchronize(st), "sync"))
        goto done;
    for (int i = 0; i < k; i++)
        energies[i] = lam[i];
    res->energy = lam[0];
    res->n_iter = xiter;
    res->n_apply_fp64 = n_fp64;
    res->n_apply_mixed = n_mixed;
    res->residual_norm2 = *std::max_element(qq.begin(), qq.begin() + k);
    if (!converged)
        rc = fail(B2G_ERR_NOT_CONVERGED, "b2g_davidson: not converged within max_iter");
    if (form == B2G_TF32X3 && b2g_heff_status(h) != B2G_OK)
        rc = B2G_ERR_STATE;
done:
    cudaStreamSynchronize(st);
    cleanup();
    return rc;
}

extern "C" int b2g_davidson(b2g_heff *h, const double *diag, double *psi, double conv_thrd,
                            int max_iter, int def_min, int def_max, int form,
                            b2g_davidson_result *res) {
    double e = 0.0;
    return davidson_impl(h, diag, psi, 1, conv_thrd, max_iter, def_min, def_max, form, &e, res);
}

extern "C" int b2g_davidson_multi(b2g_heff *h, const double *diag, double *psi, int k,
                                  double conv_thrd, int max_iter, int def_min, int def_max,
                                  int form, double *energies, b2g_davidson_result *res) {
    if (energies == nullptr)
        return fail(B2G_ERR_ARG, "b2g_davidson_multi: null energies");
    return davidson_impl(h, diag, psi, k, conv_thrd, max_iter, def_min, def_max, form, energies, res);
}
