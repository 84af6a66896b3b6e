/*
 * b2g_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's H_eff*psi replay and Davidson solver,
 * used (a) by tests as the checker of the CUDA path and (b) by bench.py's
 * cpu_baseline / --impl reference legs as the timed CPU implementation.
 * Never linked into, imported by, or called from the product path.
 *
 * b2g_oracle_replay restates BatchGEMMSeq::operator() in Tasked mode
 *   (src/core/batch_gemm.hpp:1613-1689): pairs are split statically over
 *   threads; each thread computes GEMM0 into its own work array and GEMM1
 *   into its own copy of sigma (thread 0 uses sigma itself), then the copies
 *   are summed (parallel_reduce, batch_gemm.hpp:1514-1529).  Each GEMM is the
 *   reference's single_xgemm (batch_gemm.hpp:209-235): row-major
 *   C = alpha*op(A)*op(B) + beta*C issued as a column-major dgemm with the
 *   operands swapped.  The dgemm is the BLAS named at load time (the
 *   reference links BLAS the same way, batch_gemm.hpp:57-160) or, when none
 *   is given, a plain loop nest.
 * b2g_oracle_davidson restates IterativeMatrixFunctions::davidson for one
 *   root, DavidsonTypes::Normal, Olsen preconditioner
 *   (src/core/iterative_matrix_functions.hpp:864-1173, 93-108).  The small
 *   Rayleigh-Ritz eigenproblem (LAPACK dsyev in the reference,
 *   src/core/matrix_functions.hpp:1672-1688) is solved here by cyclic Jacobi
 *   rotations; eigenvalues agree to rounding, eigenvectors up to sign.
 */
#include <dlfcn.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/b2g.h"

typedef void (*dgemm_fn)(const char *, const char *, const int *, const int *, const int *,
                         const double *, const double *, const int *, const double *, const int *,
                         const double *, double *, const int *);
static dgemm_fn g_dgemm = NULL;

/* column-major reference dgemm as a loop nest (used when no BLAS is loaded) */
static void loop_dgemm(const char *ta, const char *tb, const int *pm, const int *pn, const int *pk,
                       const double *alpha, const double *a, const int *plda, const double *b,
                       const int *pldb, const double *beta, double *c, const int *pldc) {
    const int m = *pm, n = *pn, k = *pk, lda = *plda, ldb = *pldb, ldc = *pldc;
    const int at = (*ta == 't' || *ta == 'T'), bt = (*tb == 't' || *tb == 'T');
    for (int j = 0; j < n; j++)
        for (int i = 0; i < m; i++) {
            double s = 0.0;
            for (int l = 0; l < k; l++) {
                const double x = at ? a[l + (size_t)i * lda] : a[i + (size_t)l * lda];
                const double y = bt ? b[j + (size_t)l * ldb] : b[l + (size_t)j * ldb];
                s += x * y;
            }
            double *cc = &c[i + (size_t)j * ldc];
            *cc = (*beta == 0.0 ? 0.0 : *beta * *cc) + *alpha * s;
        }
}

/* Load a BLAS providing <prefix>dgemm_ (e.g. scipy's bundled OpenBLAS with
 * prefix "scipy_"); returns 0 on success.  Threads inside BLAS are pinned to 1
 * (the reference runs BLAS single-threaded under its OpenMP loop). */
int b2g_oracle_load_blas(const char *path, const char *prefix) {
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h)
        return 1;
    char name[128];
    snprintf(name, sizeof(name), "%sdgemm_", prefix);
    g_dgemm = (dgemm_fn)dlsym(h, name);
    if (!g_dgemm)
        return 2;
    const char *setters[] = {"scipy_openblas_set_num_threads", "openblas_set_num_threads",
                             "scipy_openblas_set_num_threads64_", NULL};
    for (int i = 0; setters[i]; i++) {
        void (*f)(int) = (void (*)(int))dlsym(h, setters[i]);
        if (f) {
            f(1);
            break;
        }
    }
    return 0;
}

int b2g_oracle_blas_loaded(void) { return g_dgemm != NULL; }

/* row-major C(m x n) = alpha op(A) op(B) + beta C, as single_xgemm does it */
static inline void rm_gemm(int ta, int tb, int m, int n, int k, double alpha, const double *a,
                           int lda, const double *b, int ldb, double beta, double *c, int ldc) {
    const char *tra = ta ? "t" : "n", *trb = tb ? "t" : "n";
    dgemm_fn f = g_dgemm ? g_dgemm : loop_dgemm;
    f(trb, tra, &n, &m, &k, &alpha, b, &ldb, a, &lda, &beta, c, &ldc);
}

static int max_work_of(const b2g_pair_seq *s, size_t *out) {
    size_t mw = 0;
    for (int64_t i = 0; i < s->n_pairs; i++) {
        size_t w = (size_t)s->m0[i] * (size_t)s->n0[i];
        if (w > mw)
            mw = w;
    }
    *out = mw;
    return 0;
}

/* sigma += scale * H_eff * psi, Tasked replay with nthreads threads */
int b2g_oracle_replay(const b2g_pair_seq *s, const double *ops, const double *psi, double *sigma,
                      uint64_t sigma_size, double scale, int nthreads) {
    size_t mw;
    max_work_of(s, &mw);
    if (nthreads < 1)
        nthreads = 1;
    double **vts = (double **)calloc((size_t)nthreads, sizeof(double *));
    int err = 0;
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *v = tid == 0 ? sigma : (double *)calloc(sigma_size, sizeof(double));
        double *work = (double *)malloc(sizeof(double) * (mw ? mw : 1));
        if (!v || !work) {
#pragma omp atomic write
            err = 1;
        }
        vts[tid] = v;
        if (v && work) {
#pragma omp for schedule(static)
            for (int64_t i = 0; i < s->n_pairs; i++) {
                rm_gemm(0, s->tb0[i], s->m0[i], s->n0[i], s->k0[i], s->alpha0[i], psi + s->a0[i],
                        s->lda0[i], ops + s->b0[i], s->ldb0[i], 0.0, work, s->n0[i]);
                rm_gemm(s->ta1[i], 0, s->m1[i], s->n1[i], s->k1[i], s->alpha1[i] * scale,
                        ops + s->a1[i], s->lda1[i], work, s->n1[i], 1.0, v + s->c1[i], s->ldc1[i]);
            }
        } else {
#pragma omp for schedule(static)
            for (int64_t i = 0; i < s->n_pairs; i++) {
            }
        }
        free(work);
#pragma omp barrier
#pragma omp single
        {
            for (int t = 1; t < nthreads; t++)
                if (vts[t] && vts[0])
                    for (uint64_t j = 0; j < sigma_size; j++)
                        vts[0][j] += vts[t][j];
        }
        if (tid != 0)
            free(v);
    }
    free(vts);
    return err;
}

/* ---------------- Davidson (one root, Normal, Olsen) ---------------- */

static double vdot(const double *a, const double *b, size_t n) {
    double s = 0.0;
    for (size_t i = 0; i < n; i++)
        s += a[i] * b[i];
    return s;
}
static void vaxpy(double *y, const double *x, double a, size_t n) {
    for (size_t i = 0; i < n; i++)
        y[i] += a * x[i];
}
static void vscal(double *y, double a, size_t n) {
    for (size_t i = 0; i < n; i++)
        y[i] *= a;
}

/* symmetric eigen-decomposition by cyclic Jacobi: a (m x m, row-major, symmetric)
 * -> eigenvalues w ascending, eigenvectors as COLUMNS of v (row-major). */
int b2g_oracle_syev(int m, const double *a_in, double *w, double *v) {
    double *a = (double *)malloc(sizeof(double) * m * m);
    memcpy(a, a_in, sizeof(double) * m * m);
    for (int i = 0; i < m * m; i++)
        v[i] = 0.0;
    for (int i = 0; i < m; i++)
        v[i * m + i] = 1.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < m; i++)
            for (int j = 0; j < m; j++)
                if (i == j)
                    tot += a[i * m + j] * a[i * m + j];
                else
                    off += a[i * m + j] * a[i * m + j];
        if (off <= 1e-30 * (tot + off) || off == 0.0)
            break;
        for (int p = 0; p < m; p++)
            for (int q = p + 1; q < m; q++) {
                const double apq = a[p * m + q];
                if (apq == 0.0)
                    continue;
                const double th = (a[q * m + q] - a[p * m + p]) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < m; k++) {
                    const double akp = a[k * m + p], akq = a[k * m + q];
                    a[k * m + p] = c * akp - s * akq;
                    a[k * m + q] = s * akp + c * akq;
                }
                for (int k = 0; k < m; k++) {
                    const double apk = a[p * m + k], aqk = a[q * m + k];
                    a[p * m + k] = c * apk - s * aqk;
                    a[q * m + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < m; k++) {
                    const double vkp = v[k * m + p], vkq = v[k * m + q];
                    v[k * m + p] = c * vkp - s * vkq;
                    v[k * m + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < m; i++)
        w[i] = a[i * m + i];
    /* sort ascending (selection sort, columns follow) */
    for (int i = 0; i < m; i++) {
        int b = i;
        for (int j = i + 1; j < m; j++)
            if (w[j] < w[b])
                b = j;
        if (b != i) {
            double t = w[i];
            w[i] = w[b], w[b] = t;
            for (int k = 0; k < m; k++) {
                t = v[k * m + i];
                v[k * m + i] = v[k * m + b], v[k * m + b] = t;
            }
        }
    }
    free(a);
    return 0;
}

/*
 * One-root Davidson.  psi: initial guess in / eigenvector out.  Returns the
 * eigenvalue in *energy, iterations in *niter.  The operator is the replay of
 * the pair sequence.  Follows iterative_matrix_functions.hpp:864-1173 for k=1:
 * basis orthonormalised, sigma_i = H b_i for new vectors, Ritz problem on
 * alpha_ij = <b_i|sigma_j>, basis and sigmas rotated to Ritz vectors,
 * residual q = sigma_0 - ld_0 b_0, converged when <q|q> < conv_thrd,
 * otherwise Olsen-precondition q, restart to def_min when m reaches def_max,
 * orthogonalise q against the basis and append it.
 */
int b2g_oracle_davidson(const b2g_pair_seq *s, const double *ops, const double *diag, double *psi,
                        uint64_t n, double conv_thrd, int max_iter, int def_min, int def_max,
                        int nthreads, double *energy, int *niter) {
    if (def_min < 1)
        def_min = 1;
    if (def_max < 2)
        def_max = 2;
    double *bs = (double *)calloc((size_t)def_max * n, sizeof(double));
    double *sg = (double *)calloc((size_t)def_max * n, sizeof(double));
    double *tmp = (double *)calloc((size_t)def_max * n, sizeof(double));
    double *q = (double *)calloc(n, sizeof(double));
    double *t = (double *)calloc(n, sizeof(double));
    double *alpha = (double *)calloc((size_t)def_max * def_max, sizeof(double));
    double *ld = (double *)calloc((size_t)def_max, sizeof(double));
    double *vec = (double *)calloc((size_t)def_max * def_max, sizeof(double));
    memcpy(bs, psi, sizeof(double) * n);
    vscal(bs, 1.0 / sqrt(vdot(bs, bs, n)), n);
    int m = 1, msig = 0, xiter = 0, rc = B2G_ERR_NOT_CONVERGED;
    double qq = 0.0, e0 = 0.0;
    while (xiter < max_iter) {
        xiter++;
        for (int i = msig; i < m; i++, msig++) {
            memset(sg + (size_t)i * n, 0, sizeof(double) * n);
            b2g_oracle_replay(s, ops, bs + (size_t)i * n, sg + (size_t)i * n, n, 1.0, nthreads);
        }
        for (int i = 0; i < m; i++)
            for (int j = 0; j <= i; j++)
                alpha[i * m + j] = alpha[j * m + i] = vdot(bs + (size_t)i * n, sg + (size_t)j * n, n);
        b2g_oracle_syev(m, alpha, ld, vec);
        /* rotate: new b_j = sum_i b_i vec[i][j], same for sigma */
        memcpy(tmp, sg, sizeof(double) * m * n);
        for (int j = 0; j < m; j++) {
            double *dst = sg + (size_t)j * n;
            memset(dst, 0, sizeof(double) * n);
            for (int i = 0; i < m; i++)
                vaxpy(dst, tmp + (size_t)i * n, vec[i * m + j], n);
        }
        memcpy(tmp, bs, sizeof(double) * m * n);
        for (int j = 0; j < m; j++) {
            double *dst = bs + (size_t)j * n;
            memset(dst, 0, sizeof(double) * n);
            for (int i = 0; i < m; i++)
                vaxpy(dst, tmp + (size_t)i * n, vec[i * m + j], n);
        }
        e0 = ld[0];
        memcpy(q, sg, sizeof(double) * n);
        vaxpy(q, bs, -e0, n);
        qq = vdot(q, q, n);
        if (qq < conv_thrd) {
            rc = B2G_OK;
            break;
        }
        /* Olsen: q = K^-1 q - (c, K^-1 q)/(c, K^-1 c) K^-1 c, K = diag - ld */
        memcpy(t, bs, sizeof(double) * n);
        for (uint64_t i = 0; i < n; i++)
            if (fabs(e0 - diag[i]) > 1e-12) {
                t[i] /= e0 - diag[i];
                q[i] /= e0 - diag[i];
            }
        vaxpy(q, t, -vdot(bs, q, n) / vdot(bs, t, n), n);
        if (m >= def_max)
            m = msig = def_min;
        for (int j = 0; j < m; j++)
            vaxpy(q, bs + (size_t)j * n, -vdot(bs + (size_t)j * n, q, n), n);
        vscal(q, 1.0 / sqrt(vdot(q, q, n)), n);
        memcpy(bs + (size_t)m * n, q, sizeof(double) * n);
        m++;
    }
    memcpy(psi, bs, sizeof(double) * n);
    *energy = e0;
    *niter = xiter;
    free(bs), free(sg), free(tmp), free(q), free(t), free(alpha), free(ld), free(vec);
    return rc;
}
