// Perturbative noise as GEMM pairs (host only).
//
// EffectiveHamiltonian::perturbative_noise (src/dmrg/effective_hamiltonian.hpp:262-433)
// applies the left or right half of H_eff to the converged ket: in Tasked mode
// block2 records it as single GEMMs in BatchGEMMSeq::batch[1]
// (BatchGEMMSeq::multiply and three_rotate_tr_left/right,
// src/core/batch_gemm.hpp:887-891, 1025-1107; the per-row form of
// AdvancedGEMM::multiply, batch_gemm.hpp:584-607), each
//   c (m x n, ld ldc) += alpha op_a(A) op_b(B)
// with one operand a block of the ket and the other an operator block, c a
// block of the perturbed-wavefunction group.  The H_eff engine replays GEMM
// pairs (W = psi_blk op(B0); sigma += alpha op(A1) W), so each GEMM becomes
// one pair with an identity block on the side it lacks:
//   ket on the left:   W = ket_blk op_b(B)   c += alpha I_m W
//   ket on the right:  W = ket_blk I_n       c += alpha op_a(A) W
// Products with an identity block are exact in FP64 (every other term is an
// exact zero), so the pair replay equals the GEMM list up to summation order.
#include <algorithm>
#include <string>
#include <vector>

#include "b2g_internal.h"

namespace b2g {
namespace {

// stored extent (doubles) of op(X) with logical shape rows x cols and leading dimension ld
uint64_t stored_extent(bool t, int64_t rows, int64_t cols, int64_t ld) {
    if (rows == 0 || cols == 0)
        return 0;
    return t ? (uint64_t)((cols - 1) * ld + rows) : (uint64_t)((rows - 1) * ld + cols);
}

// off + ext <= size, in a form no offset can make wrap around
bool fits(uint64_t off, uint64_t ext, uint64_t size) { return ext <= size && off <= size - ext; }

} // namespace
} // namespace b2g

using namespace b2g;

extern "C" int b2g_noise_pairs(const b2g_gemm_list *g, uint64_t ket_size, uint64_t ops_size,
                               uint64_t group_size, int64_t n_blocks, const uint64_t *blk_off,
                               const int32_t *blk_rows, const int32_t *blk_cols, b2g_pair_arrays *out,
                               int64_t *n_pairs, int32_t *id_dim) {
    if (g == nullptr || out == nullptr || n_pairs == nullptr || id_dim == nullptr || g->n_gemms < 0 ||
        n_blocks < 0 || (n_blocks > 0 && (blk_off == nullptr || blk_rows == nullptr || blk_cols == nullptr)))
        return fail(B2G_ERR_ARG, "b2g_noise_pairs: null or negative argument");
    if (g->n_gemms > 0) {
        const void *in[] = {g->ta, g->tb, g->m, g->n, g->k, g->lda, g->ldb, g->ldc, g->a_kind, g->b_kind,
                            g->alpha, g->beta, g->a, g->b, g->c};
        const void *outp[] = {out->tb0, out->m0, out->n0, out->k0, out->lda0, out->ldb0, out->ta1, out->m1,
                              out->n1, out->k1, out->lda1, out->ldc1, out->alpha0, out->alpha1, out->a0,
                              out->b0, out->a1, out->c1};
        for (const void *x : in)
            if (x == nullptr)
                return fail(B2G_ERR_ARG, "b2g_noise_pairs: null GEMM-list array");
        for (const void *x : outp)
            if (x == nullptr)
                return fail(B2G_ERR_ARG, "b2g_noise_pairs: null pair array");
    }
    for (int64_t b = 0; b < n_blocks; b++) {
        const uint64_t sz = (uint64_t)std::max(blk_rows[b], 0) * (uint64_t)std::max(blk_cols[b], 0);
        if (blk_rows[b] < 0 || blk_cols[b] < 0 || !fits(blk_off[b], sz, group_size) ||
            (b > 0 && blk_off[b] < blk_off[b - 1]))
            return fail(B2G_ERR_ARG, "b2g_noise_pairs: group block " + std::to_string(b) +
                                         " out of range or out of order");
    }
    const std::string where = "b2g_noise_pairs: GEMM ";
    std::vector<char> id_b0, id_a1;  // pair reads the identity as its GEMM0 B / GEMM1 A
    int64_t np = 0;
    int32_t dim = 0;
    for (int64_t q = 0; q < g->n_gemms; q++) {
        bool ta = g->ta[q] != 0, tb = g->tb[q] != 0;
        int64_t m = g->m[q], n = g->n[q], k = g->k[q];
        int64_t lda = g->lda[q], ldb = g->ldb[q], ldc = g->ldc[q];
        int32_t akind = g->a_kind[q], bkind = g->b_kind[q];
        uint64_t a = g->a[q], b = g->b[q];
        const uint64_t c = g->c[q];
        const double alpha = g->alpha[q];
        if (m < 0 || n < 0 || k < 0)
            return fail(B2G_ERR_ARG, where + std::to_string(q) + " has a negative dimension");
        if (g->beta[q] != 1.0)
            return fail(B2G_ERR_ARG, where + std::to_string(q) + " has beta != 1 (not an accumulation)");
        if ((akind != B2G_NOISE_KET && akind != B2G_NOISE_OP) || (bkind != B2G_NOISE_KET && bkind != B2G_NOISE_OP) ||
            akind == bkind)
            return fail(B2G_ERR_ARG, where + std::to_string(q) + " does not have exactly one ket operand");
        if (m == 0 || n == 0 || k == 0 || alpha == 0.0)
            continue;
        if (lda < (ta ? m : k) || ldb < (tb ? k : n) || ldc < n)
            return fail(B2G_ERR_ARG, where + std::to_string(q) + " has a leading dimension below its row length");
        if (!fits(a, stored_extent(ta, m, k, lda), akind == B2G_NOISE_KET ? ket_size : ops_size) ||
            !fits(b, stored_extent(tb, k, n, ldb), bkind == B2G_NOISE_KET ? ket_size : ops_size) ||
            !fits(c, stored_extent(false, m, n, ldc), group_size))
            return fail(B2G_ERR_ARG, where + std::to_string(q) + " reads or writes out of range");
        if (bkind == B2G_NOISE_KET && tb) {
            // the per-row form: c (m x 1, contiguous) = op_a(A) b^T with b one ket row;
            // as a whole, c^T (1 x m) = b op_a(A)^T
            if (n != 1 || ldc != 1)
                return fail(B2G_ERR_UNSUPPORTED, where + std::to_string(q) +
                                                     " has a transposed ket operand and a non-vector output");
            std::swap(a, b), std::swap(akind, bkind);
            const bool new_tb = !ta;
            ldb = lda, tb = new_tb, ta = false, lda = k;
            n = m, m = 1, ldc = n;
        }
        if (akind == B2G_NOISE_KET && ta) {
            // a transposed k x 1 column with leading dimension 1 is one contiguous row
            if (m != 1 || lda != 1)
                return fail(B2G_ERR_UNSUPPORTED, where + std::to_string(q) +
                                                     " has a transposed ket operand that is not one row");
            ta = false, lda = k;
        }
        // the output's group block: a one-row output takes the block's leading dimension
        const int64_t blk = (int64_t)(std::upper_bound(blk_off, blk_off + n_blocks, c) - blk_off) - 1;
        if (blk < 0)
            return fail(B2G_ERR_UNSUPPORTED, where + std::to_string(q) + " writes outside the group blocks");
        const int64_t cols = blk_cols[blk];
        const uint64_t rel = c - blk_off[blk];
        if (m == 1)
            ldc = cols;
        if (cols == 0 || ldc != cols || (int64_t)(rel % (uint64_t)cols) + n > cols ||
            rel / (uint64_t)cols + (uint64_t)m > (uint64_t)blk_rows[blk])
            return fail(B2G_ERR_UNSUPPORTED, where + std::to_string(q) + " output leaves its group block");
        if (akind == B2G_NOISE_KET) {  // W = ket_blk (m x k) op_b(B);  c += alpha I_m W
            out->tb0[np] = tb, out->m0[np] = (int32_t)m, out->n0[np] = (int32_t)n, out->k0[np] = (int32_t)k;
            out->lda0[np] = (int32_t)lda, out->ldb0[np] = (int32_t)ldb, out->a0[np] = a, out->b0[np] = b;
            out->ta1[np] = 0, out->m1[np] = (int32_t)m, out->n1[np] = (int32_t)n, out->k1[np] = (int32_t)m;
            out->a1[np] = ops_size;
            id_b0.push_back(0), id_a1.push_back(1);
            dim = std::max(dim, (int32_t)m);
        } else {                       // W = ket_blk (k x n) I_n;  c += alpha op_a(A) (m x k) W
            out->tb0[np] = 0, out->m0[np] = (int32_t)k, out->n0[np] = (int32_t)n, out->k0[np] = (int32_t)n;
            out->lda0[np] = (int32_t)ldb, out->a0[np] = b, out->b0[np] = ops_size;
            out->ta1[np] = ta, out->m1[np] = (int32_t)m, out->n1[np] = (int32_t)n, out->k1[np] = (int32_t)k;
            out->lda1[np] = (int32_t)lda, out->a1[np] = a;
            id_b0.push_back(1), id_a1.push_back(0);
            dim = std::max(dim, (int32_t)n);
        }
        out->ldc1[np] = (int32_t)ldc, out->c1[np] = c;
        out->alpha0[np] = 1.0, out->alpha1[np] = alpha;
        np++;
    }
    for (int64_t p = 0; p < np; p++) {
        if (id_b0[p])
            out->ldb0[p] = dim;
        if (id_a1[p])
            out->lda1[p] = dim;
    }
    *n_pairs = np;
    *id_dim = dim;
    return B2G_OK;
}
