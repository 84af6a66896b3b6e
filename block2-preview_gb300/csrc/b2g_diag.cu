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
// sub-block).  The plan builder cuts each sigma region into tiles of
// kDiagTileRows x kDiagTileCols cells and lists, per tile, the contributions
// whose sigma rectangle meets the tile on rows where their psi and sigma
// sub-blocks overlap -- no other contribution can reach a diagonal cell there.
// One CTA per tile, one thread per tile column; a thread owns the column's
// cells and loops over the tile's list in contribution order for each of
// them (no atomics, reproducible; tiles are disjoint, so every cell has one
// owner).  The list is staged through shared memory in chunks; each entry
// carries the frame position of its psi sub-block, so the psi index of a cell
// needs no division.
#include <algorithm>

#include "b2g_internal.h"

namespace b2g {

namespace {

constexpr int kDiagChunk = 128;   // contributions staged in shared memory at a time

__global__ void __launch_bounds__(kDiagTileCols) diag_kernel(const DiagTask *__restrict__ tasks,
                                                             const int32_t *__restrict__ tlist,
                                                             const DiagItem *__restrict__ items,
                                                             const Region *__restrict__ regions,
                                                             const double *__restrict__ ops,
                                                             double *__restrict__ diag) {
    __shared__ DiagItem si[kDiagChunk];
    const DiagTask t = tasks[blockIdx.x];
    const Region rg = regions[t.g];
    const int c = t.c0 + (int)threadIdx.x;
    const bool col_ok = c < t.c1;
    double s[kDiagTileRows];
    bool covered[kDiagTileRows];
#pragma unroll
    for (int q = 0; q < kDiagTileRows; q++)
        s[q] = 0.0, covered[q] = false;
    for (int64_t e0 = t.lb; e0 < t.le; e0 += kDiagChunk) {
        const int n = (int)min((int64_t)kDiagChunk, t.le - e0);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            si[i] = items[tlist[e0 + i]];
        __syncthreads();
        if (!col_ok)
            continue;
        for (int e = 0; e < n; e++) {
            const DiagItem &it = si[e];
            const int j = c - it.col0;
            if (j < 0 || j >= it.n1)
                continue;
            // the psi column l of cell column c (and the row shift when the psi
            // window wraps the frame), row-independent
            int l = c - it.ca, kshift = 0;
            if (l < 0)
                l += rg.ld, kshift = 1;
#pragma unroll
            for (int q = 0; q < kDiagTileRows; q++) {
                const int r = t.r0 + q;
                const int i = r - it.row0;
                if (r >= t.r1 || i < 0 || i >= it.m1)
                    continue;
                covered[q] = true;
                uint64_t k, lu;
                if (it.same_ld) {
                    const int kk = r - it.ra - kshift;
                    if (kk < 0 || kk >= it.m0 || l >= it.k0)
                        continue;
                    k = (uint64_t)kk, lu = (uint64_t)l;
                } else {
                    const uint64_t x = rg.base + (uint64_t)r * rg.ld + (uint64_t)c;
                    if (x < it.a0)
                        continue;
                    const uint64_t dy = x - it.a0;
                    k = dy / (uint64_t)it.lda0, lu = dy % (uint64_t)it.lda0;
                    if (k >= (uint64_t)it.m0 || lu >= (uint64_t)it.k0)
                        continue;
                }
                const double lv = ops[it.a1 + (it.ta1 ? k * it.lda1 + i : (uint64_t)i * it.lda1 + k)];
                const double rv = ops[it.b0 + (it.tb0 ? (uint64_t)j * it.ldb0 + lu : lu * it.ldb0 + j)];
                s[q] = fma(it.alpha * lv, rv, s[q]);
            }
        }
    }
    if (!col_ok)
        return;
#pragma unroll
    for (int q = 0; q < kDiagTileRows; q++) {
        const int r = t.r0 + q;
        if (r >= t.r1 || !covered[q])
            continue;
        const uint64_t x = rg.base + (uint64_t)r * rg.ld + (uint64_t)c;
        if (x < rg.lo || x >= rg.hi)
            continue;
        diag[x] += s[q];
    }
}

} // namespace

cudaError_t launch_diag(const DevicePlan &p, const double *ops, double *diag, cudaStream_t s) {
    if (p.n_diag_task == 0)
        return cudaSuccess;
    if (p.n_diag_task > 0x7fffffff)
        return cudaErrorInvalidConfiguration;
    note_launch();
    diag_kernel<<<(unsigned)p.n_diag_task, kDiagTileCols, 0, s>>>(p.diag_task, p.diag_tlist, p.diag_item,
                                                                   p.regions, ops, diag);
    return cudaGetLastError();
}

} // namespace b2g
