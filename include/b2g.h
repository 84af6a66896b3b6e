/*
 * b2g.h -- C ABI of the GB300 (sm_103a) two-site DMRG hot path.
 *
 * The library replaces, behind block2's own C++ API, the part of a two-site
 * DMRG sweep where the time goes: the block-sparse effective-Hamiltonian
 * product H_eff*psi replayed every Davidson iteration, the Davidson
 * eigensolver around it.
 *
 * Boundary (reference interfaces each entry point replaces):
 *   b2g_heff_create   <- EffectiveHamiltonian::precompute, which records the
 *                        GEMM pairs of one H_eff*psi into BatchGEMMSeq
 *                        (src/dmrg/effective_hamiltonian.hpp:226-246,
 *                         src/core/batch_gemm.hpp:893-902 rotate,
 *                         src/core/batch_gemm.hpp:952-1065 three_rotate)
 *   b2g_heff_apply    <- BatchGEMMSeq::operator()(c, v, scale) in Tasked mode
 *                        (src/core/batch_gemm.hpp:1570-1690), reached through
 *                        TensorFunctions::operator() (src/core/tensor_functions.hpp:59-62)
 *   b2g_heff_apply_host  same, with host buffers (H2D psi, D2H sigma inside)
 *   b2g_heff_destroy  <- EffectiveHamiltonian::post_precompute / deallocate
 *                        (src/dmrg/effective_hamiltonian.hpp:247-253)
 *   b2g_davidson      <- IterativeMatrixFunctions::davidson, Normal type,
 *                        Olsen preconditioner
 *                        (src/core/iterative_matrix_functions.hpp:864-1173, 93-108)
 *                        as called by EffectiveHamiltonian::eigs
 *                        (src/dmrg/effective_hamiltonian.hpp:481-568)
 *   (further entries below: diag, multi-root products and Davidson, density-
 *    matrix truncation, environment blocking, quantum-number bookkeeping and
 *    connection infos, term partition, the perturbative-noise product as
 *    GEMM pairs; and, without a reference counterpart, the adjoint of
 *    H_eff*psi, the tile autotuner and the allocation-free product -- each
 *    with the interface it replaces or the reason it exists)
 *
 * Conventions: row-major matrices (as GMatrix, src/core/matrix.hpp:94-106);
 * offsets and sizes count doubles; every function returns 0 on success and a
 * B2G_ERR_* code otherwise, with a message in b2g_last_error() (the C++ shim
 * turns a non-zero status into std::runtime_error, the reference's error
 * convention).  No torch or C++ types cross this boundary.
 */
#ifndef B2G_H
#define B2G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define B2G_OK 0
#define B2G_ERR_ARG 1          /* invalid argument / inconsistent sequence */
#define B2G_ERR_CUDA 2         /* CUDA runtime error */
#define B2G_ERR_NOMEM 3        /* device allocation failed */
#define B2G_ERR_UNSUPPORTED 4  /* sequence shape the plan builder cannot take */
#define B2G_ERR_NOT_CONVERGED 5/* Davidson reached max_iter */
#define B2G_ERR_STATE 6        /* wrong call order / destroyed object */

/* arithmetic forms of H_eff*psi */
#define B2G_FP64 0             /* plain FP64 (CUDA-core DFMA) */
#define B2G_TF32X3 1           /* split-TF32 x3 on tcgen05 tensor cores, FP32 accumulate */
#define B2G_FP32 2             /* FP32 on CUDA cores (FFMA), FP32 accumulate */

/*
 * The recorded GEMM-pair sequence of one H_eff*psi: BatchGEMMSeq::batch[0]
 * (GEMM0) and batch[1] (GEMM1) after EffectiveHamiltonian::precompute, one
 * entry per pair, struct-of-arrays, with every pointer replaced by an offset:
 * a0 into psi (precompute sets cmat->data = 0), b0/a1 into the packed operator
 * blob, c1 into sigma (vmat->data = 0).  Pair i computes
 *
 *   W  = alpha0[i] * psi[a0:](m0 x k0, ld lda0) * op_b0(ops[b0:])(k0 x n0, ld ldb0)
 *   sigma[c1:](m1 x n1, ld ldc1) += scale * alpha1[i] * op_a1(ops[a1:])(m1 x k1, ld lda1) * W
 *
 * with op_b0 = transpose when tb0[i] != 0, op_a1 = transpose when ta1[i] != 0,
 * and k1 == m0, n1 == n0 (W is the per-pair work matrix of
 * AdvancedGEMM::rotate, src/core/batch_gemm.hpp:564-575).
 */
typedef struct {
    int64_t n_pairs;
    const int32_t *tb0, *m0, *n0, *k0, *lda0, *ldb0;
    const int32_t *ta1, *m1, *n1, *k1, *lda1, *ldc1;
    const double *alpha0, *alpha1;
    const uint64_t *a0, *b0, *a1, *c1;
} b2g_pair_seq;

typedef struct b2g_context b2g_context;
typedef struct b2g_heff b2g_heff;

typedef struct {
    int64_t n_pairs;        /* recorded pairs */
    int64_t n_work;         /* distinct GEMM0 products after de-duplication */
    int64_t n_regions;      /* disjoint sigma regions (atomic-free owners) */
    int64_t n_tiles;        /* GEMM1 output tiles launched per apply */
    double mnk;             /* reference multiply-add count: sum m0 n0 k0 + m1 n1 k1 */
    double mnk_executed;    /* multiply-adds the plan executes (after de-duplication) */
    uint64_t ops_bytes;     /* operator blob bytes resident in HBM */
    uint64_t work_bytes;    /* GEMM0 work buffer bytes */
    uint64_t plan_bytes;    /* schedule tables bytes */
    uint64_t psi_size, sigma_size;
} b2g_heff_stats;

/* version and error reporting */
int b2g_version(void);
const char *b2g_last_error(void);
/* Kernels this library has launched in this process so far (a replayed CUDA
 * graph counts the kernels it holds).  No reference counterpart: launch
 * accounting for measurements. */
int b2g_launch_count(uint64_t *out);

/* one context per device (the device is made current by every call) */
int b2g_context_create(int device, b2g_context **out);
int b2g_context_destroy(b2g_context *ctx);
/* the CUDA stream the context launches on (cudaStream_t), for callers that sync/overlap */
void *b2g_context_stream(b2g_context *ctx);
/* A pinned (page-locked) host buffer of at least `bytes` owned by the context,
 * for staging operator blobs: host->device copies from it run at the link's
 * full rate and without driver staging.  The pointer stays valid until a
 * later call asks for more bytes (the buffer is then replaced, after the
 * context stream has drained) or the context is destroyed.  No reference
 * counterpart (block2's operators live in its own pageable allocators). */
int b2g_host_buffer(b2g_context *ctx, uint64_t bytes, void **out);
int b2g_context_synchronize(b2g_context *ctx);

/*
 * Build the device plan of one H_eff from its recorded pair sequence and
 * upload the operator blob (ops_size doubles; host memory when
 * ops_on_device == 0, else a device pointer that is copied).  With
 * ops_on_device == B2G_OPS_DEFERRED the blob is allocated but not filled
 * (ops may be NULL): the caller installs the values with b2g_heff_set_ops
 * before the first product, e.g. while this call builds the plan on another
 * thread.
 */
#define B2G_OPS_DEFERRED 2
int b2g_heff_create(b2g_context *ctx, const b2g_pair_seq *seq, const double *ops,
                    uint64_t ops_size, int ops_on_device, uint64_t psi_size,
                    uint64_t sigma_size, b2g_heff **out);
int b2g_heff_destroy(b2g_heff *h);
int b2g_heff_stats_get(const b2g_heff *h, b2g_heff_stats *out);
/* Synchronizes the context stream and reports B2G_ERR_STATE if a
 * tensor-core kernel of this H_eff gave up a bounded wait (its result is
 * then incomplete).  b2g_heff_apply_host and b2g_davidson check this too. */
int b2g_heff_status(b2g_heff *h);
/* Host-only dry run of the plan builder (no device touched): validates the
 * sequence against the sizes and reports the schedule statistics. */
int b2g_plan_stats(const b2g_pair_seq *seq, uint64_t ops_size, uint64_t psi_size,
                   uint64_t sigma_size, b2g_heff_stats *out);
/* Host-only term partition of one H_eff over n_ranks ranks.  Replaces the
 * reference's term distribution (ParallelRuleQC, src/dmrg/qc_parallel_rule.hpp:31-85)
 * whose partial sigmas ParallelTensorFunctions::operator() sums with
 * allreduce_sum (src/core/parallel_tensor_functions.hpp:51-55).  Pairs sharing
 * a GEMM0 product stay on one rank; products go largest first to the
 * least-loaded rank (ties: lower rank, earlier product), so every rank derives
 * the same partition.  rank_of_pair[i] receives the rank of pair i; load
 * (optional, n_ranks doubles) the multiply-adds each rank executes.  Each rank
 * builds b2g_heff_create from its own pairs and sums sigma across ranks. */
int b2g_partition_pairs(const b2g_pair_seq *seq, int n_ranks, int32_t *rank_of_pair,
                        double *load);

/* sigma += scale * H_eff * psi; psi and sigma are DEVICE pointers (sizes as created),
 * form = B2G_FP64 or B2G_TF32X3.  Asynchronous on the context stream. */
int b2g_heff_apply(b2g_heff *h, const double *psi, double *sigma, double scale, int form);
/* same with HOST psi/sigma: copies psi in, applies, copies sigma out, synchronizes. */
int b2g_heff_apply_host(b2g_heff *h, const double *psi, double *sigma, double scale, int form);
/* sigma_r += scale * H_eff * psi_r for nroots right-hand sides stored one after
 * another (psi: nroots * psi_size, sigma: nroots * sigma_size, DEVICE pointers),
 * in one launch per kernel.  Replaces the one-vector-at-a-time application of
 * state-averaged effective Hamiltonians (EffectiveHamiltonian<..., MultiMPS>
 * ::operator(), src/dmrg/effective_hamiltonian.hpp:1690, and
 * TensorFunctions::tensor_product_multi_multiply, src/core/tensor_functions.hpp:806-870). */
int b2g_heff_apply_batch(b2g_heff *h, const double *psi, double *sigma, int nroots, double scale,
                         int form);

/*
 * diag(H_eff) in FP64 (the Davidson preconditioner), computed on the device
 * from the recorded pairs: entry x collects, over the pairs whose sigma block
 * holds x, alpha0 * alpha1 * op(L)[i][k] * op(R)[l][j] for the psi index
 * y = x.  Replaces the diagonal the reference builds in the EffectiveHamiltonian
 * constructor (src/dmrg/effective_hamiltonian.hpp:190-200, via
 * TensorFunctions::tensor_product_diagonal, src/core/tensor_functions.hpp:2027-2183).
 * diag: sigma_size doubles, a DEVICE pointer (b2g_heff_diag, asynchronous) or a
 * HOST pointer (b2g_heff_diag_host, synchronous).  Needs psi_size == sigma_size.
 */
int b2g_heff_diag(b2g_heff *h, double *diag);
int b2g_heff_diag_host(b2g_heff *h, double *diag);

/*
 * Environment blocking: the operators of the enlarged block, built from the
 * environment operators and the site operators by the reference's
 * TensorFunctions::left_contract / right_contract
 * (src/core/tensor_functions.hpp:2842-2986), given as block-level records:
 *   iadd  (OperatorFunctions::iadd, src/core/operator_functions.hpp:135-170):
 *         tmp[dst](m x n) += f * op(blob_src[src])      (op = transpose if conj;
 *         blob 0 = env, 1 = site)
 *   kron  (OperatorFunctions::tensor_product, operator_functions.hpp:672-710,
 *         GMatrixFunctions::tensor_product, src/core/matrix_functions.hpp:1269):
 *         out[c + (i bm' + k) cn + j bn' + l] += f * A'(i,j) * B'(k,l),
 *         A' = op(blob_a[a]) (am x an stored, transposed if ca), B' likewise,
 *         blobs 0 = env, 1 = site, 2 = the iadd intermediates.
 * out (out_size doubles) is overwritten with the sum of the kron records; all
 * iadd records are applied before any kron record.  Host buffers; FP64.
 */
typedef struct {
    int64_t n_iadd;
    const int32_t *ia_m, *ia_n, *ia_conj, *ia_src_blob;
    const uint64_t *ia_dst, *ia_src;
    const double *ia_f;
    int64_t n_kron;
    const int32_t *kr_am, *kr_an, *kr_ca, *kr_bm, *kr_bn, *kr_cb, *kr_cn, *kr_ablob, *kr_bblob;
    const uint64_t *kr_a, *kr_b, *kr_c;
    const double *kr_f;
} b2g_block_seq;

int b2g_block_contract(b2g_context *ctx, const b2g_block_seq *seq, const double *env,
                       uint64_t env_size, const double *site, uint64_t site_size,
                       uint64_t tmp_size, double *out, uint64_t out_size);
/* The same with env, site and out as DEVICE pointers (the environment stays
 * resident between sites: the output can feed b2g_heff_create with
 * ops_on_device = 1 or the next blocking without a host round trip). */
int b2g_block_contract_device(b2g_context *ctx, const b2g_block_seq *seq, const double *env,
                              uint64_t env_size, const double *site, uint64_t site_size,
                              uint64_t tmp_size, double *out, uint64_t out_size);

/*
 * sigma += scale * H_eff * psi in plain FP64 without allocating anything.
 * No counterpart in the reference: this entry point exists for callers that
 * cannot call cudaMalloc (a program that hands the GPU a fixed memory budget,
 * or code running where an allocation would synchronize the device or break
 * its memory accounting).  The caller passes the recorded pair sequence
 * (host arrays), and DEVICE pointers to the operator blob, psi and sigma;
 * the work matrices live in a 32 MiB file-scope device array that every GPU
 * loading this library holds until exit.  A pair whose work matrix exceeds
 * that array is rejected (B2G_ERR_ARG).  Calls share the array, so calls
 * that overlap on the GPU race.  The call must not be captured into a CUDA
 * graph: each chunk's pair descriptors are copied from one host array owned
 * by the library, which the next chunk or call overwrites, so a replay would
 * run on stale descriptors.
 * sigma is accumulated with FP64 atomics, so unlike the other FP64 entry
 * points the result is not bit-reproducible from call to call (it differs
 * in the last bits).  The pair descriptors reach the device through an
 * ordinary copy from pageable host memory, so a call can hold the host
 * until that copy is staged.
 * stream: a cudaStream_t (NULL = legacy default stream).  Asynchronous.
 */
int b2g_heff_apply_noalloc(const b2g_pair_seq *seq, const double *ops, uint64_t ops_size,
                           const double *psi, uint64_t psi_size, double *sigma,
                           uint64_t sigma_size, double scale, void *stream);

/*
 * Differentiation form (the adjoint of H_eff*psi).  No counterpart in the
 * reference, which obtains energy derivatives only as reduced density
 * matrices from its expectation sweeps (src/dmrg/sweep_algorithm.hpp,
 * class Expect); the adjoint follows the pair semantics of
 * BatchGEMMSeq::rotate (src/core/batch_gemm.hpp:893-902).
 *
 * b2g_heff_set_ops: replace the operator values of an H_eff (same layout and
 *   size as created; host pointer when ops_on_device == 0, else a device
 *   pointer that is copied).  The reduced-precision copies follow.
 * b2g_heff_adjoint_prepare: build the adjoint schedule from the sequence the
 *   H_eff was created from (host work, device tables and work matrices).
 * b2g_heff_adjoint: for bra x (sigma_size) and ket y (psi_size), DEVICE
 *   pointers, with f = <x| H_eff(ops) |y>:
 *     grad_ops[i] += scale * df/dops[i]   (ops_size doubles, may be NULL)
 *     grad_psi[j] += scale * df/dy[j] = scale * (H_eff^T x)[j]  (psi_size, may be NULL)
 *   FP64, deterministic (no atomics), asynchronous on the context stream.
 *   The gradient buffers must not overlap x, y or each other.
 * b2g_heff_adjoint_mnk: multiply-adds of one adjoint with both gradients.
 */
int b2g_heff_set_ops(b2g_heff *h, const double *ops, int ops_on_device);
int b2g_heff_adjoint_prepare(b2g_heff *h, const b2g_pair_seq *seq);
int b2g_heff_adjoint(b2g_heff *h, const double *x, const double *y, double scale, double *grad_ops,
                     double *grad_psi);
int b2g_heff_adjoint_mnk(const b2g_heff *h, double *mnk);

/* Per-kernel timing of b2g_heff_apply (CUDA events recorded on the context
 * stream around each phase when enabled; no work is skipped).  ms[0] =
 * GEMM0 phase, ms[1] = GEMM1 phase of the most recent apply (synchronizes). */
int b2g_heff_set_timing(b2g_heff *h, int enable);
int b2g_heff_last_timing(b2g_heff *h, float *ms);

/* CUDA-graph replay of repeated applies (on by default).  The reference
 * replays its recorded BatchGEMMSeq on every Davidson iteration
 * (src/core/batch_gemm.hpp:1570-1690); here the first apply with a given
 * (psi, sigma, nroots, scale, form) runs its kernels directly, the second is
 * captured into a CUDA graph and replayed, later ones replay it (at most 64
 * graphs per H_eff, least recently used dropped; growing the root count drops
 * them all).  Timing mode bypasses the graphs.  enable = 0 drops every graph. */
int b2g_heff_set_graphs(b2g_heff *h, int enable);
/* number of captured graphs held (-1 for a null handle) */
int b2g_heff_graph_count(const b2g_heff *h);

/* Autotuner of the tensor-core tile shapes (no reference counterpart: the
 * reference's BatchGEMMSeq replays fixed MKL calls).  From the block-size
 * histogram of this H_eff's plan it lists candidate shapes -- GEMM0 tiles of
 * 256 or 128 stacked psi rows (128 only tried when some right operator is
 * shared by more rows), GEMM1 tiles of 256 or 128 sigma columns (128 only
 * when some rectangle is wider), split-K chunks of 32, 64 or 16 K slabs -- times
 * one TF32x3 apply of each (median of 5 after 2 warm-ups, L2 flushed between
 * applies) and keeps the fastest plan installed.  seq must be the sequence
 * the H_eff was created from.  Only form = B2G_TF32X3 has tile shapes. */
typedef struct {
    int32_t n_candidates, best;     /* candidates timed; index of the kept one */
    float ms[12];                   /* median apply time per candidate */
    int32_t g0_tile_cols[12], g1_tile_cols[12], g1_chunk[12];
    double g1_wide_frac;            /* GEMM1 stage work in tiles wider than 128 columns */
    double g0_wide_frac;            /* GEMM0 tiles with more than 128 stacked rows */
} b2g_tune_result;
int b2g_heff_autotune(b2g_heff *h, const b2g_pair_seq *seq, int form, b2g_tune_result *res);
/* tile shapes of the installed plan: params[0] GEMM0 tile rows, params[1]
 * GEMM1 tile columns, params[2] split-K chunk length */
int b2g_heff_get_params(const b2g_heff *h, int32_t *params);
/* install the plan with the given tile shapes (same meaning; 128 or 256, 128
 * or 256, 1..64) without timing, e.g. shapes an earlier autotune kept */
int b2g_heff_set_params(b2g_heff *h, const b2g_pair_seq *seq, const int32_t *params);

/* Measured compute ceiling of one arithmetic form on this device (a
 * register-resident FMA/MMA loop, no memory traffic), in TFLOP/s; used as
 * the roofline denominator for forms without a measured copy or GEMM peak (FP64).
 * form = B2G_FP64: FP64 FMA on the CUDA cores (DFMA); B2G_PROBE_FP64_MMA: the
 * FP64 tensor-core instruction (mma.sync m8n8k4 f64, DMMA). */
#define B2G_PROBE_FP64_MMA 16
int b2g_probe_peak(b2g_context *ctx, int form, double *tflops);

/*
 * Davidson for the lowest eigenpair of H_eff (one root), the reference's
 * Normal Davidson with Olsen preconditioning and thick restart to
 * def_min vectors when def_max is reached.  diag: diag(H_eff) (host),
 * psi: initial guess in, converged eigenvector out (host).  Convergence on
 * |r|^2 < conv_thrd.  form selects the arithmetic of the H_eff products that
 * expand the basis; for a reduced-precision form (B2G_TF32X3, B2G_FP32)
 * convergence is only ever declared on an FP64 residual: when the subspace
 * residual is small, one FP64 product on the Ritz vector x gives the exact
 * r = Hx - (x,Hx)x; if |r|^2 >= conv_thrd the basis restarts from x with its
 * exact sigma and continues (defect correction).  The energy returned is
 * the FP64 Rayleigh quotient.  Outputs: energy (eigenvalue, without
 * const_e), iterations, number of H_eff products by form.
 */
typedef struct {
    double energy;
    int32_t n_iter;
    int32_t n_apply_fp64;
    int32_t n_apply_mixed;
    double residual_norm2;
} b2g_davidson_result;

int b2g_davidson(b2g_heff *h, const double *diag, double *psi, double conv_thrd,
                 int max_iter, int def_min, int def_max, int form,
                 b2g_davidson_result *res);

/*
 * The k lowest eigenpairs (state-averaged roots; the reference's davidson
 * with k = vs.size() > 1, src/core/iterative_matrix_functions.hpp:864-1173, as
 * used by EffectiveHamiltonian<..., MultiMPS>::eigs,
 * src/dmrg/effective_hamiltonian.hpp:1711-1797).  psi: k guesses in, k
 * eigenvectors out (host, k * psi_size); energies: k eigenvalues.  Block
 * variant: each iteration adds the Olsen corrections of all unconverged roots
 * and computes their H_eff products in one b2g_heff_apply_batch call; the
 * reduced-precision forms certify every root on FP64 residuals.
 */
int b2g_davidson_multi(b2g_heff *h, const double *diag, double *psi, int k, double conv_thrd,
                       int max_iter, int def_min, int def_max, int form, double *energies,
                       b2g_davidson_result *res);

/*
 * Block layout of a two-site wavefunction and of its reduced density matrix.
 * psi block a is psi_rows[a] x psi_cols[a], row-major at psi_off[a]; it
 * contributes to density-matrix block psi_dm[a] (-1: none), which is square
 * of size dm_dim[b].  trace_right != 0 traces out the right index (forward
 * sweep: rho_b = sum_a psi_a psi_a^T over row quanta), else the left index
 * (rho_b = sum_a psi_a^T psi_a over column quanta).  This is the mapping
 * OperatorFunctions::trans_product applies, src/core/operator_functions.hpp:
 * 777-838.
 */
typedef struct {
    int32_t trace_right;
    int32_t n_psi_blocks;
    const int32_t *psi_dm;
    const int32_t *psi_rows;
    const int32_t *psi_cols;
    const uint64_t *psi_off;
    int32_t n_dm_blocks;
    const int32_t *dm_dim;
} b2g_dm_layout;

typedef struct {
    double error;   /* discarded weight: sum of the positive discarded eigenvalues */
    int32_t n_kept; /* states kept over all blocks */
} b2g_dm_result;

/*
 * Density-matrix truncation of one two-site step, FP64:
 * MovingEnvironment::density_matrix (without noise) + split_density_matrix
 * with TruncationTypes::Physical (src/dmrg/moving_environment.hpp:3554-3580,
 * 3715-3843, 4250-4345).  rho is formed and diagonalised on the device;
 * the k largest eigenvalues are kept (k = -1 keeps all), then trailing kept
 * states below cutoff are dropped while more than one remains.
 * Host buffers:
 *   psi       the wavefunction (layout above)
 *   eigvals   out, sum(dm_dim): each block's eigenvalues, ascending
 *   kept      out, n_dm_blocks: states kept per block
 *   rotation  out, room for sum(dm_dim^2): per block with kept[b] > 0, in
 *             block order, the kept eigenvectors in ascending eigenvalue
 *             order -- trace_right: dm_dim x kept (vectors as columns, the
 *             left MPS tensor); else kept x dm_dim (vectors as rows, the
 *             right MPS tensor)
 *   wfn       out, room for the psi length: per psi block whose dm block
 *             keeps states, in psi block order -- trace_right: rot^T psi_a
 *             (kept x psi_cols); else psi_a rot^T (psi_rows x kept) -- the
 *             whole scaled to unit norm (the reference's normalize = true)
 * Returns B2G_ERR_UNSUPPORTED for a density-matrix block above 4000 states,
 * B2G_ERR_NOT_CONVERGED if a QL iteration needs more than 60 steps.
 */
int b2g_dm_truncate(b2g_context *ctx, const b2g_dm_layout *layout, const double *psi, int k,
                    double cutoff, double *eigvals, int32_t *kept, double *rotation,
                    double *wfn, b2g_dm_result *res);

/* ---- Quantum-number bookkeeping (host only, bit-exact with the reference) ----
 * Labels are the reference's packed 64-bit words: SZLongLong
 * (src/core/symmetry.hpp:656, N | 2Sz | pg) and SU2LongLong
 * (src/core/symmetry.hpp:1185, N | 2S_low | 2S | pg).  A StateInfo is n
 * ascending labels with their state counts (src/core/state_info.hpp:60-200). */
#define B2G_SYM_SZ 0
#define B2G_SYM_SU2 1
/* b2g_quanta_op operations (symmetry.hpp operator+, unary -, count, [k],
 * get_ket, get_bra, combine): out = a + b | -a | a.count() | a[b] | a.get_ket()
 * | a.get_bra(b) | a.combine(bra = b, ket = c) (a is the delta quantum). */
#define B2G_QOP_ADD 0
#define B2G_QOP_NEG 1
#define B2G_QOP_COUNT 2
#define B2G_QOP_ELEM 3
#define B2G_QOP_KET 4
#define B2G_QOP_BRA 5
#define B2G_QOP_COMBINE 6
typedef struct {
    int32_t n;           /* labels (on output: count; on input of an output: capacity) */
    uint64_t *quanta;    /* n packed labels, ascending */
    uint32_t *n_states;  /* n state counts */
} b2g_state_info;

int b2g_quanta_op(int sym, int op, uint64_t a, uint64_t b, uint64_t c, uint64_t *out);
/* StateInfo::tensor_product (state_info.hpp:231-276): every coupled label of
 * a x b; with cref != NULL only labels of cref are kept (counts added into
 * cref's slots), otherwise labels above target are dropped; counts saturate
 * at ubond_max (65535 for the reference's default 16-bit ubond_t).  c->n is
 * the capacity on entry and the label count on return. */
int b2g_state_tensor_product(int sym, uint32_t ubond_max, const b2g_state_info *a,
                             const b2g_state_info *b, const b2g_state_info *cref,
                             uint64_t target, b2g_state_info *c);
/* StateInfo::get_connection_info (state_info.hpp:280-307): for each label of
 * c the (i, j) label pairs of a and b that couple to it; acc (c->n + 1)
 * offsets into ij (pairs stored as i, j; capacity cap pairs). */
int b2g_state_connection(int sym, const b2g_state_info *a, const b2g_state_info *b,
                         const b2g_state_info *c, uint32_t *acc, uint32_t *ij, int64_t cap,
                         int64_t *n_pairs);
/* SparseMatrixInfo::initialize (sparse_matrix.hpp:727-757) of an operator
 * (wfn = 0) or wavefunction (wfn = 1) with delta quantum dq between bra and
 * ket, plus initialize_block_shifts / get_total_memory (sparse_matrix.hpp:
 * 617-630, 804-820) with 32-bit offsets and blocks rounded up to align
 * elements (1 unless the reference runs with an AlignTypes alignment). */
int b2g_wfn_blocks(int sym, const b2g_state_info *bra, const b2g_state_info *ket, uint64_t dq,
                   int wfn, uint32_t align, uint64_t *quanta, uint32_t *rows, uint32_t *cols,
                   uint32_t *shifts, int cap, int *n_blocks, uint32_t *total);

/* Operator infos of one side of an H_eff (left_op_infos / right_op_infos of
 * the EffectiveHamiltonian constructor): n infos sorted by delta quantum, each
 * with its fermion flag and its ascending block labels quanta[start[i] ..
 * start[i + 1]). */
typedef struct {
    int32_t n;
    const uint64_t *dq;
    const int32_t *fermion;
    const int32_t *start;
    const uint64_t *quanta;
} b2g_op_infos;
/* ConnectionInfo::initialize_wfn (sparse_matrix.hpp:163-292), as the
 * EffectiveHamiltonian constructor calls it (effective_hamiltonian.hpp:208-216):
 * for each sub-label k (sub_conj[k] in 0..3: bit 0 left operator transposed,
 * bit 1 right; sub_q[k] its label) and each bra block, the coupled (left op
 * block, right op block, ket block) triples with their Clebsch-Gordan factor
 * (SU(2): 9j symbol x transposition factors x fermion sign; SZ: sign only).
 * Outputs: n5 (5 conj-type boundaries), idx (n_sub starts), and nc entries of
 * stride (bra block), factor, ia, ib, ic (capacity cap). */
int b2g_wfn_connection(int sym, uint64_t cdq, uint64_t vdq, uint64_t opdq, int32_t n_sub,
                       const int32_t *sub_conj, const uint64_t *sub_q, const b2g_op_infos *left,
                       const b2g_op_infos *right, int32_t n_ket, const uint64_t *ket_q, int32_t n_bra,
                       const uint64_t *bra_q, int32_t *n5, uint32_t *idx, uint64_t *stride,
                       double *factor, uint32_t *ia, uint32_t *ib, uint32_t *ic, int64_t cap,
                       int64_t *nc);

/*
 * Perturbative noise (EffectiveHamiltonian::perturbative_noise,
 * src/dmrg/effective_hamiltonian.hpp:262-433, called from
 * DMRG::two_dot_eigs_and_perturb, src/dmrg/sweep_algorithm.hpp:1257-1260).
 * In Tasked mode block2 records that product as single GEMMs in
 * BatchGEMMSeq::batch[1] (BatchGEMMSeq::multiply, three_rotate_tr_left/right,
 * src/core/batch_gemm.hpp:887-891, 1025-1107; the per-row form of
 * AdvancedGEMM::multiply, batch_gemm.hpp:584-607), each, row-major,
 *
 *   group[c:](m x n, ld ldc) += alpha * op_a(A)(m x k) * op_b(B)(k x n)
 *
 * (beta = 1), one operand a block of the ket (kind B2G_NOISE_KET, offset into
 * the ket), the other an operator block (B2G_NOISE_OP, offset into the
 * operator blob), c an offset into the perturbed-wavefunction group.
 */
#define B2G_NOISE_KET 0
#define B2G_NOISE_OP 1
typedef struct {
    int64_t n_gemms;
    const int32_t *ta, *tb, *m, *n, *k, *lda, *ldb, *ldc;
    const int32_t *a_kind, *b_kind;
    const double *alpha, *beta;
    const uint64_t *a, *b, *c;
} b2g_gemm_list;
/* Writable pair arrays (the fields of b2g_pair_seq), capacity n_gemms each. */
typedef struct {
    int32_t *tb0, *m0, *n0, *k0, *lda0, *ldb0;
    int32_t *ta1, *m1, *n1, *k1, *lda1, *ldc1;
    double *alpha0, *alpha1;
    uint64_t *a0, *b0, *a1, *c1;
} b2g_pair_arrays;
/*
 * Rewrites a noise GEMM list as the GEMM pairs of b2g_pair_seq over
 * psi = the ket, sigma = the group, and the operator blob followed by an
 * identity block, so that b2g_heff_create / b2g_heff_apply run it.  No
 * reference counterpart (block2 replays the list with its batched BLAS):
 *   ket on the left:   W = ket_blk op_b(B),  c += alpha I W
 *   ket on the right:  W = ket_blk I,        c += alpha op_a(A) W
 * (products with the identity are exact in FP64).  A transposed ket operand is
 * accepted where it is one contiguous row; a GEMM whose transposed ket row is
 * its B operand (output one contiguous column) is transposed as a whole.
 * The caller appends the row-major identity block (*id_dim x *id_dim) at
 * offset ops_size of the blob.  Group layout: n_blocks row-major blocks in
 * ascending order, block i at blk_off[i] with blk_rows[i] x blk_cols[i]
 * elements; a one-row output takes its block's leading dimension.  GEMMs with
 * a zero dimension or alpha = 0 are dropped.  Outputs: *n_pairs pairs in out,
 * *id_dim.  B2G_ERR_ARG: an operand out of range, beta != 1, not exactly one
 * ket operand; B2G_ERR_UNSUPPORTED: a transposed ket operand that is not one
 * row, an output that leaves its group block.  Host only.
 */
int b2g_noise_pairs(const b2g_gemm_list *g, uint64_t ket_size, uint64_t ops_size,
                    uint64_t group_size, int64_t n_blocks, const uint64_t *blk_off,
                    const int32_t *blk_rows, const int32_t *blk_cols, b2g_pair_arrays *out,
                    int64_t *n_pairs, int32_t *id_dim);

#ifdef __cplusplus
}
#endif

#endif /* B2G_H */
