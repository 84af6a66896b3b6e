// Internal types of the GB300 DMRG hot-path library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/b2g.h"

namespace b2g {

void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

// Kernel-launch accounting (b2g_launch_count): every launch site calls
// note_launch(); launches made while a stream capture is being recorded on
// this thread count towards the graph being built instead, and each replay of
// a captured graph adds the kernels it holds.
void note_launch(uint64_t n = 1);
void capture_begin();
uint64_t capture_end();   // kernels recorded since capture_begin()

#define B2G_CUDA_TRY(expr)                                                                  \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess)                                                              \
            return ::b2g::fail(B2G_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)

// ---------------------------------------------------------------------------
// Device plan of one H_eff (built once per site from the recorded pairs).
//
// Phase 1 (GEMM0, de-duplicated): distinct products W_u = psi[a0:] * op(ops[b0:])
//   are computed once each into the work buffer; one warp per row of W_u.
// Phase 2 (GEMM1, atomic-free): sigma is partitioned into disjoint regions
//   (the sigma blocks the pairs write); each region is cut into tasks of
//   4 rows x up to 256 columns, each task owns its cells and loops over the
//   list of pair contributions alpha * op(A1) * W_u that overlap its rows.
// ---------------------------------------------------------------------------
struct WorkDesc {       // one distinct GEMM0 product
    uint64_t a0, b0, woff;
    int32_t m0, n0, k0, lda0, ldb0, tb0;
};
struct Contrib {        // one GEMM1 contribution (one recorded pair)
    uint64_t a1;        // operator offset
    double alpha;       // alpha0 * alpha1
    int32_t u;          // work product index
    int32_t row0, col0; // placement inside the region
    int32_t m1, n1, k1, lda1, ta1;
};
struct Region {
    uint64_t base;      // sigma offset of (0, 0)
    uint64_t lo, hi;    // merged write span [lo, hi): cells owned by this region
    int32_t ld, rows, cols, pad;
};
struct Task1 {          // phase 1: one row of one work product
    int32_t u, r;
};
// phase 2: rows [4*rb, 4*rb+4) x cols [col0, col0+256) of a region, one chunk of
// its contribution list (split-K over chunks of at most kSimtChunkK k-steps)
constexpr int kSimtChunkK = 768;
struct Task2 {
    int32_t g, rb, col0, chunk;
    int64_t lb, le;     // contribution list range of this chunk
    int64_t part;       // partial-tile slot (in 4 x 256 tiles) of chunk 0, -1: single chunk
};
// diag(H_eff): one tile (rows [r0, r1) x columns [c0, c1)) of region g and
// the diagonal contributions that can reach a cell of it, diag_tlist[lb ..
// le), in contribution order (tiles are disjoint: one owner per diagonal cell)
struct DiagTask {
    int32_t g, r0, r1, c0, c1, pad;
    int64_t lb, le;
};
// one contribution that can reach diag(H_eff), in its region's frame: the
// diagonal cell (r, c) (flat x = base + r ld + c) takes alpha op(L)[i][k]
// op(R)[l][j] with i = r - row0, j = c - col0 and x - a0 = k lda0 + l.  When
// the psi sub-block lies in a block with the region's row stride (lda0 = ld,
// always so for a square H_eff: overlapping psi and sigma sub-blocks are in
// one wavefunction block), x - a0 = (r - ra) ld + (c - ca) and (k, l) follow
// without a division (same_ld = 1).
struct DiagItem {
    uint64_t a1, b0, a0;    // op(L) / op(R) block offsets in the blob, psi offset
    double alpha;           // alpha0 * alpha1
    int32_t row0, col0, m1, n1;   // sigma rectangle in the frame
    int32_t ra, ca;         // frame row / column of a0 (0 <= ca < ld) when same_ld
    int32_t m0, k0, lda0, lda1, ldb0;
    int16_t ta1, tb0;
    int32_t same_ld, pad;
};
constexpr int kDiagTileCols = 256;     // columns per tile (one per thread)
constexpr int kDiagTileRows = 8;       // rows per tile
struct Tile2 {          // a phase-2 tile split over several chunks (reduced after)
    int32_t g, rb, col0, n_chunks;
    int64_t part;
};

// Tensor-core stages are 16 K columns (two K = 8 MMA steps).  FP32
// accumulation in TMEM over very long K loses accuracy, so the GEMM1 chunks
// end after at most kTcMaxChunkStages stages (512 K) and the FP64 reduction
// sums the chunks.
constexpr int kTcStageK = 16;
constexpr int kTcMaxChunkStages = 32;
constexpr int kG1ChunkLimit = 64;   // longest chunk the GEMM1 kernel's stage table holds

// Tensor-core GEMM0 of the TF32x3 form, transposed: W_u^T = op(R)^T *
// psi_u^T for the distinct products sharing one right operator block R.  A
// tile is one 128-row piece of op(R)^T (rows = columns of W, M) times up to
// 256 stacked psi rows of those products (N; each product's rows padded to a
// multiple of 4), K = k0 in 16-column slabs.  The R piece comes from a static
// operator image (bulk copies), the psi rows are gathered per stage, and the
// epilogue writes the accumulator straight into the W images GEMM1 reads
// (every 4 stacked columns are one 16-byte K chunk of one W image row).
struct G0Tile {
    uint64_t a;                 // byte offset of slab 0 of the op(R)^T image piece
    uint32_t a_bytes;           // rows8 * 64: one split part of one slab
    int32_t nsl;                // K slabs
    int32_t rows, n, ncol;      // valid M rows (<= 128), MMA N (multiple of 16), valid columns
    int32_t k0, npad, m_off;    // K, W image width (n0 rounded up to 16), W column of row 0
    int64_t cb;                 // first entry in the column table
};
struct G0Psi {                  // one distinct psi sub-block, packed per product
    uint64_t src;               // psi offset (a0)
    uint64_t dst;               // packed offset (floats, multiple of 4)
    int32_t m0, k0, lda0, k0p;  // rows, columns, psi leading dimension, packed row stride (k0 -> 4)
};
struct G0Col {                  // one stacked psi row (one W image K row)
    uint64_t psi;               // packed-psi offset of the row (16-byte aligned)
    uint64_t w;                 // byte offset of its W image (per root)
    int32_t k;                  // row index i within the product
    int32_t live;               // i < m0 (padding rows read zeros)
};

// Image-fed tensor-core GEMM1 (the TF32x3 form's sigma phase).  The
// contributions of a region are grouped by their sigma rectangle (rows
// [row0, row0 + m1) x cols [col0, col0 + n1) of the region frame); a tile is
// one 128-row x <=256-column piece of a rectangle, so every stage of a tile
// fills the same accumulator rows.  Operands live in HBM already split into
// TF32 hi/lo parts and laid out as the canonical no-swizzle K-major tiles the
// MMA reads (8-row x 16-byte core matrices, 512 B between 8-row groups for a
// 16-column K slab):
//   A images (static per H_eff): alpha * op(L) of each distinct (block,
//     alpha), per 128-row piece and 16-column slab [hi: rows8 x 64 B | lo];
//   W images (per product, from the GEMM0 output): W_u^T per 16-row slab of
//     W_u, [hi: npad x 64 B | lo: npad x 64 B], npad = n0 rounded up to 16.
// A stage is one slab of one contribution: two bulk copies of A (hi, lo) and
// two of B, then three MMAs per K = 8 half.  Every tile chunk stores a
// partial tile; the reduction sums, per sigma cell, the partials of all the
// tiles covering it in a fixed order (rectangles of one region may overlap).
struct G1Tile {
    int32_t g, row0, col0;      // region and origin (region frame)
    int32_t rows, n, n_chunks;  // valid rows (<= 128), MMA width (multiple of 16, <= 256), chunks
    int32_t ncols, pad;         // valid columns (<= n)
    int64_t part;               // offset (floats) of chunk 0's partial tile
};
struct G1Stage {
    uint64_t a;                 // byte offset of the A hi slab (lo follows after a_bytes)
    uint64_t b;                 // byte offset of the B hi slab (per root, in the W image buffer)
    uint32_t a_bytes;           // rows8 * 64
    uint32_t b_lo;              // byte distance hi -> lo in the B image (npad * 64)
};
struct G1Task {
    int32_t tile, chunk;
    int64_t st0;                // first stage
    int32_t n_stages, pad;
};
struct G1AImg {                 // one A image to build: alpha * op(L), all pieces and slabs
    uint64_t src;               // operator offset (floats)
    uint64_t dst;               // byte offset of the image
    float alpha;
    int32_t m1, k1, lda1, ta1, pad;
};
struct G1WImg {                 // one W image per distinct GEMM0 product
    uint64_t dst;               // byte offset (per root)
    int32_t u, npad;            // work product, padded width
};
struct G1Red {                  // reduction item: rows [r0, r1) of region g
    int32_t g, r0, r1, t0;      // tile list [t0, t1) of the region (cover list)
    int32_t t1, pad;
};
constexpr int kG1SlabK = 16;

// tile shapes of the tensor-core form (the autotuner's search space)
struct PlanParams {
    int32_t g0_tile_cols = 256;              // stacked psi rows per GEMM0 tile (128 or 256)
    int32_t g1_tile_cols = 256;              // sigma columns per GEMM1 tile (128 or 256)
    int32_t g1_chunk = kTcMaxChunkStages;    // K slabs per GEMM1 split-K chunk (<= kG1ChunkLimit)
};

struct HostPlan {
    PlanParams params;
    std::vector<G0Tile> g0tile;
    std::vector<G0Col> g0col;
    std::vector<G0Psi> g0psi;
    int64_t g0_wide = 0;            // tiles [0, g0_wide) are wider than 128 columns
    uint64_t g0_psi_floats = 0;     // packed psi floats per root
    std::vector<WorkDesc> works;
    std::vector<Contrib> contribs;
    std::vector<Region> regions;
    std::vector<int64_t> region_cb;  // contributions of region g: [region_cb[g], region_cb[g + 1])
    // contributions whose psi sub-block overlaps their sigma sub-block (the
    // only ones that can reach diag(H_eff)), listed per row band of each region
    std::vector<DiagTask> diag_task;
    std::vector<int32_t> diag_tlist;    // indices into diag_item
    std::vector<DiagItem> diag_item;
    std::vector<Task1> t1;
    std::vector<Task2> t2;
    std::vector<Tile2> t2multi;
    uint64_t t2_part_tiles = 0;     // 4 x 256 partial tiles of split phase-2 tiles
    std::vector<int32_t> lists;
    uint64_t work_size = 0;
    double mnk = 0, mnk_exec = 0;
    // image-fed tensor-core GEMM1
    std::vector<G1Tile> g1tile;
    std::vector<G1Stage> g1stage;
    std::vector<G1Task> g1task;
    std::vector<G1AImg> g1aimg;
    std::vector<G1WImg> g1wimg;
    std::vector<G1Red> g1red;
    std::vector<int32_t> g1cover;   // tile ids per region (reduction cover lists)
    uint64_t g1_abytes = 0;         // A image bytes
    uint64_t g1_wbytes = 0;         // W image bytes per root
    uint64_t g1_part = 0;           // partial floats per root
};

int build_plan(const b2g_pair_seq *seq, uint64_t ops_size, uint64_t psi_size, uint64_t sigma_size,
               HostPlan &plan, const PlanParams &params = PlanParams());

struct DevicePlan {
    WorkDesc *works = nullptr;
    Contrib *contribs = nullptr;
    Region *regions = nullptr;
    int64_t *region_cb = nullptr;
    DiagTask *diag_task = nullptr;
    int32_t *diag_tlist = nullptr;
    DiagItem *diag_item = nullptr;
    int64_t n_diag_task = 0;
    Task1 *t1 = nullptr;
    Task2 *t2 = nullptr;
    Tile2 *t2multi = nullptr;
    int64_t n_t2multi = 0;
    int32_t *lists = nullptr;
    G0Tile *g0tile = nullptr;
    G0Col *g0col = nullptr;
    G0Psi *g0psi = nullptr;
    int64_t n_g0tile = 0, n_g0psi = 0, n_g0wide = 0;  // tiles [0, n_g0wide) are wider than 128
    uint64_t g0_psi_floats = 0;
    int64_t n_works = 0, n_contribs = 0, n_regions = 0, n_t1 = 0, n_t2 = 0, n_lists = 0;
    G1Tile *g1tile = nullptr;
    G1Stage *g1stage = nullptr;
    G1Task *g1task = nullptr;
    G1AImg *g1aimg = nullptr;
    G1Red *g1red = nullptr;
    int32_t *g1cover = nullptr;
    int64_t n_g1task = 0, n_g1aimg = 0, n_g1red = 0;
    uint64_t g1_abytes = 0, g1_wbytes = 0, g1_part = 0;
};

// Several right-hand sides (roots) in one launch: root r (blockIdx.y) reads
// psi + r * psi, writes sigma + r * sigma, and uses its own slice of the work
// and split-K partial buffers (strides in elements of the buffer's type).
struct RootStrides {
    int nroots = 1;
    uint64_t psi = 0, sigma = 0, work = 0, part = 0;
    uint64_t wimg = 0;   // W image bytes per root (image-fed GEMM1)
};

// tensor-core launchers (b2g_tc.cu); err: device int set non-zero when a
// bounded wait gives up
cudaError_t launch_g0(const DevicePlan &p, const unsigned char *aimg, const double *psi,
                      float *psi_packed, unsigned char *wimg, int *err, const RootStrides &rs,
                      cudaStream_t s);

// image-fed tensor-core GEMM1 (b2g_g1.cu)
cudaError_t launch_g1_build_a(const DevicePlan &p, const float *ops32, unsigned char *aimg,
                              cudaStream_t s);
cudaError_t launch_g1(const DevicePlan &p, const unsigned char *aimg, const unsigned char *wimg,
                      float *part, double *sigma, double scale, int *err, const RootStrides &rs,
                      cudaStream_t s);

// diag(H_eff) from the recorded pairs (b2g_diag.cu), FP64, device output
cudaError_t launch_diag(const DevicePlan &p, const double *ops, double *diag, cudaStream_t s);

// CUDA-core launchers (b2g_simt.cu), T = double (FP64 form) or float (FP32 form)
template <typename T>
cudaError_t launch_simt_phase1(const DevicePlan &p, const T *ops, const T *psi, T *work,
                               const RootStrides &rs, cudaStream_t s);
template <typename T>
cudaError_t launch_simt_phase2(const DevicePlan &p, const T *ops, const T *work, double *sigma,
                               T *part, double scale, const RootStrides &rs, cudaStream_t s);
cudaError_t launch_to_float(const double *x, float *y, uint64_t n, cudaStream_t s);
// compute-ceiling probe: TFLOP/s of a register-resident FP64 FMA loop
cudaError_t probe_fp64_peak(cudaStream_t s, int n_sm, double *tflops);
cudaError_t probe_fp64_mma_peak(cudaStream_t s, int n_sm, double *tflops);

} // namespace b2g

struct b2g_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    int n_sm = 0;
    void *host_buf = nullptr;     // pinned staging buffer (b2g_host_buffer)
    uint64_t host_buf_bytes = 0;
};

namespace b2g {
// one captured H_eff*psi (CUDA graph) for a fixed argument set: the second
// apply with the same psi, sigma, root count, scale and form captures its
// launches, later ones replay the graph
struct ApplyGraph {
    const double *psi = nullptr;
    double *sigma = nullptr;
    int nroots = 0, form = 0;
    double scale = 0.0;
    cudaGraphExec_t exec = nullptr;
    uint64_t n_kernels = 0;  // kernels the captured graph launches
    int state = 0;        // 0 seen once, 1 captured, -1 not capturable (runs eagerly)
    uint64_t last = 0;    // LRU tick
};
constexpr size_t kMaxApplyGraphs = 64;
struct AdjointPlan;   // the adjoint's schedule and work matrices (b2g_adjoint.cu)
} // namespace b2g

struct b2g_heff {
    b2g_context *ctx = nullptr;
    b2g::DevicePlan plan;
    double *ops = nullptr;
    float *ops32 = nullptr;  // operators rounded to float (made on the first reduced-precision apply)
    float *psi32 = nullptr;  // psi rounded to float (per reduced-precision apply)
    double *work = nullptr;  // cap_roots x work_size doubles (FP32 forms use it as floats)
    double *psi_stage = nullptr, *sigma_stage = nullptr; // device staging for the host entry
    void *simt_part = nullptr;   // cap_roots x phase-2 partial tiles (doubles)
    unsigned char *g1_aimg = nullptr;  // A images (made with ops32)
    unsigned char *g1_wimg = nullptr;  // g1_roots x W images
    float *g1_part = nullptr;          // g1_roots x image-fed GEMM1 partial tiles
    int g1_roots = 0;                  // roots the W images / partials are sized for
    float *g0_psi = nullptr;           // g1_roots x packed psi sub-blocks (GEMM0 operand)
    int cap_roots = 0;           // roots the per-root buffers are sized for
    int stage_roots = 0;         // roots the host staging buffers are sized for
    uint64_t ops_size = 0, psi_size = 0, sigma_size = 0, work_size = 0;
    uint64_t simt_part_size = 0;  // per root, in elements
    b2g_heff_stats stats{};
    bool timing = false;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    int *err = nullptr;     // device flag: a bounded wait in a tensor-core kernel gave up
    b2g::PlanParams params;  // tile shapes of the installed plan
    bool graphs_on = true;  // replay repeated applies as CUDA graphs
    std::vector<b2g::ApplyGraph> graphs;
    uint64_t graph_tick = 0;
    b2g::AdjointPlan *adj = nullptr;  // made by b2g_heff_adjoint_prepare
};

namespace b2g {
void free_adjoint(b2g_heff *h);
} // namespace b2g
