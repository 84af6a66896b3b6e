// Diagonal of H_eff (the Davidson preconditioner) from the recorded GEMM pairs.
//
// The reference computes diag(H_eff) while building the effective Hamiltonian
// (EffectiveHamiltonian ctor, src/dmrg/effective_hamiltonian.hpp:190-200,
// through TensorFunctions::tensor_product_diagonal,
// src/core/tensor_functions.hpp:2027-2183, whose per-block kernel adds
// diag(op(L)) x diag(op(R)): OperatorFunctions::tensor_product_diagonal,
// src/core/operator_functions.hpp:211-247, and AdvancedGEMM
// ::tensor_product_diagonal, src/core/batch_gemm.hpp:689-703).  The same
// numbers follow from the pair list H_eff*psi replays: pair p maps psi[y] to
// sigma[x] with coefficient alpha0 alpha1 op(L)[i][k] op(R)[l][j], where
// x = c1 + i ldc1 + j and y = a0 + k lda0 + l, so the diagonal entry x
// collects, over the pairs whose sigma block holds x, the term with y = x
// (k = (x - a0) / lda0, l = (x - a0) % lda0, when that lands inside the psi
// sub-block).  The plan builder cuts each sigma region into row bands of about
// kDiagBandCells cells and lists, per band, the contributions whose psi and
// sigma sub-blocks overlap on rows of that band -- every other contribution
// cannot reach a diagonal cell there.  One CTA per band; one thread owns a
// cell and loops over the band's list in contribution order (no atomics,
// reproducible; bands are disjoint, so every cell has one owner).
#include <algorithm>

#include "b2g_internal.h"

namespace b2g {

namespace {

__global__ void __launch_bounds__(256) diag_kernel(const DiagTask *__restrict__ tasks,
                                                   const int32_t *__restrict__ tlist,
                                                   const Region *__restrict__ regions,
                                                   const Contrib *__restrict__ contribs,
                                                   const WorkDesc *__restrict__ works,
                                                   const double *__restrict__ ops,
                                                   double *__restrict__ diag) {
    const DiagTask t = tasks[blockIdx.x];
    const Region rg = regions[t.g];
    const int64_t ncell = (int64_t)(t.r1 - t.r0) * rg.cols;
    for (int64_t cell = threadIdx.x; cell < ncell; cell += blockDim.x) {
        const int r = t.r0 + (int)(cell / rg.cols), c = (int)(cell % rg.cols);
        const uint64_t x = rg.base + (uint64_t)r * rg.ld + (uint64_t)c;
        if (x < rg.lo || x >= rg.hi)
            continue;
        double s = 0.0;
        bool covered = false;
        for (int64_t e = t.lb; e < t.le; e++) {
            const Contrib ct = contribs[tlist[e]];
            const int i = r - ct.row0, j = c - ct.col0;
            if (i < 0 || i >= ct.m1 || j < 0 || j >= ct.n1)
                continue;
            covered = true;
            const WorkDesc w = works[ct.u];
            if (x < w.a0)
                continue;
            const uint64_t dy = x - w.a0;
            const uint64_t k = dy / (uint64_t)w.lda0, l = dy % (uint64_t)w.lda0;
            if (k >= (uint64_t)w.m0 || l >= (uint64_t)w.k0)
                continue;
            const double lv = ops[ct.a1 + (ct.ta1 ? k * ct.lda1 + i : (uint64_t)i * ct.lda1 + k)];
            const double rv = ops[w.b0 + (w.tb0 ? (uint64_t)j * w.ldb0 + l : l * w.ldb0 + j)];
            s = fma(ct.alpha * lv, rv, s);
        }
        if (covered)
            diag[x] += s;
    }
}

} // namespace

cudaError_t launch_diag(const DevicePlan &p, const double *ops, double *diag, cudaStream_t s) {
    if (p.n_diag_task == 0)
        return cudaSuccess;
    if (p.n_diag_task > 0x7fffffff)
        return cudaErrorInvalidConfiguration;
    note_launch();
    diag_kernel<<<(unsigned)p.n_diag_task, 256, 0, s>>>(p.diag_task, p.diag_tlist, p.regions, p.contribs,
                                                         p.works, ops, diag);
    return cudaGetLastError();
}

} // namespace b2g
