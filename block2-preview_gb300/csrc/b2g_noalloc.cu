// H_eff*psi (plain FP64) for callers that must not allocate device memory.
//
// Who needs this: code that runs where cudaMalloc is off limits -- a host
// program that hands the GPU a fixed memory budget up front (its own pool or
// arena, a real-time or embedded loop), or a caller sitting inside a region
// where an allocation would synchronize the device or break its memory
// accounting.  Such a caller owns psi, sigma and the operator blob on the
// device and passes them in; this entry point adds no allocation of its own.
//
// How: the per-pair work matrices and the pair descriptors live in one
// file-scope device array, kNoAllocScratchBytes (32 MiB) large, that every
// GPU which loads this library holds until the process exits.  Pairs are
// processed in chunks that fit the array (descriptors copied in, GEMM0 into
// the array, GEMM1 accumulated into sigma with FP64 atomics, so the order of
// the additions into one sigma element varies between runs and the FP64
// result can differ in its last bits from call to call).
//
// Rules for callers:
//   * the first call on a device looks up the device address of the array
//     (cudaGetSymbolAddress) with that device current;
//   * no call may be captured into a CUDA graph: the descriptors are copied
//     from one host staging array that the next chunk or call overwrites, so
//     a replay would run on stale descriptors;
//   * every call shares the one array and leaves the last chunk's contents in
//     it; calls whose work overlaps on the GPU (different streams, or
//     different host threads on one device) race on it -- serialize them;
//   * a single pair whose work matrix does not fit the array is rejected with
//     B2G_ERR_ARG before anything is launched;
//   * each chunk's descriptors go from a host staging array to the device by
//     an ordinary cudaMemcpyAsync from pageable memory, so a call can hold
//     the host until that copy has been staged.
#include <mutex>

#include "b2g_internal.h"

namespace b2g {

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;
constexpr int kMaxDevices = 64;
constexpr int kChunkPairs = 4096;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NaPair {
    uint64_t a0, b0, a1, c1, woff;
    double alpha0, alpha1;
    int32_t m0, n0, k0, lda0, ldb0, tb0;
    int32_t m1, n1, k1, lda1, ldc1, ta1;
};

// descriptors of one chunk, staged on the host (no heap use)
static NaPair g_host_desc[kChunkPairs];
static std::mutex g_mu;
static void *g_dev_scratch[kMaxDevices] = {};

constexpr size_t kDescBytes = sizeof(NaPair) * kChunkPairs;
constexpr size_t kWorkDoubles = (kNoAllocScratchBytes - kDescBytes) / sizeof(double);

// one CTA per pair: W = alpha0 * psi_sub * op(B)
__global__ void na_gemm0(const NaPair *__restrict__ d, const double *__restrict__ ops,
                         const double *__restrict__ psi, double *__restrict__ work) {
    const NaPair p = d[blockIdx.x];
    double *W = work + p.woff;
    for (int e = threadIdx.x; e < p.m0 * p.n0; e += blockDim.x) {
        const int r = e / p.n0, c = e % p.n0;
        double s = 0.0;
        for (int k = 0; k < p.k0; k++) {
            const double b = p.tb0 ? ops[p.b0 + (uint64_t)c * p.ldb0 + k]
                                   : ops[p.b0 + (uint64_t)k * p.ldb0 + c];
            s = fma(psi[p.a0 + (uint64_t)r * p.lda0 + k], b, s);
        }
        W[e] = p.alpha0 * s;
    }
}

// one CTA per pair: sigma_sub += scale * alpha1 * op(A) * W  (FP64 atomics)
__global__ void na_gemm1(const NaPair *__restrict__ d, const double *__restrict__ ops,
                         const double *__restrict__ work, double *sigma, double scale) {
    const NaPair p = d[blockIdx.x];
    const double *W = work + p.woff;
    const double f = scale * p.alpha1;
    for (int e = threadIdx.x; e < p.m1 * p.n1; e += blockDim.x) {
        const int r = e / p.n1, c = e % p.n1;
        double s = 0.0;
        for (int k = 0; k < p.k1; k++) {
            const double a = p.ta1 ? ops[p.a1 + (uint64_t)k * p.lda1 + r]
                                   : ops[p.a1 + (uint64_t)r * p.lda1 + k];
            s = fma(a, W[(uint64_t)k * p.n1 + c], s);
        }
        atomicAdd(sigma + p.c1 + (uint64_t)r * p.ldc1 + c, f * s);
    }
}

// device address of the scratch array for the current device (looked up once)
int scratch_address(int dev, unsigned char **out) {
    if (dev < 0 || dev >= kMaxDevices)
        return fail(B2G_ERR_ARG, "b2g_heff_apply_noalloc: device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_dev_scratch[dev] == nullptr) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr)
            return fail(B2G_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                          cudaGetErrorString(e));
        g_dev_scratch[dev] = p;
    }
    *out = (unsigned char *)g_dev_scratch[dev];
    return B2G_OK;
}

} // namespace

} // namespace b2g

using namespace b2g;

extern "C" int b2g_heff_apply_noalloc(const b2g_pair_seq *seq, const double *ops, uint64_t ops_size,
                                      const double *psi, uint64_t psi_size, double *sigma,
                                      uint64_t sigma_size, double scale, void *stream) {
    if (seq == nullptr || (seq->n_pairs > 0 && (ops == nullptr || psi == nullptr || sigma == nullptr)))
        return fail(B2G_ERR_ARG, "b2g_heff_apply_noalloc: null argument");
    // validation of every pair (same rules as the plan builder), before any launch
    for (int64_t i = 0; i < seq->n_pairs; i++) {
        const int64_t m0 = seq->m0[i], n0 = seq->n0[i], k0 = seq->k0[i];
        const int64_t m1 = seq->m1[i], n1 = seq->n1[i], k1 = seq->k1[i];
        if (m0 < 0 || n0 < 0 || k0 < 0 || m1 < 0 || n1 < 0 || k1 < 0)
            return fail(B2G_ERR_ARG, "b2g_heff_apply_noalloc: negative dimension");
        if (k1 != m0 || n1 != n0)
            return fail(B2G_ERR_UNSUPPORTED, "b2g_heff_apply_noalloc: GEMM1 does not consume GEMM0");
        if (m1 == 0 || n1 == 0 || k1 == 0 || k0 == 0)
            continue;
        // a row must fit its leading dimension (op(X) stored rows x cols)
        if (seq->lda0[i] < k0 || seq->ldb0[i] < (seq->tb0[i] ? k0 : n0) ||
            seq->lda1[i] < (seq->ta1[i] ? m1 : k1) || seq->ldc1[i] < n1)
            return fail(B2G_ERR_ARG, "b2g_heff_apply_noalloc: pair " + std::to_string(i) +
                                         " has a leading dimension below its row length");
        auto ext = [](bool t, int64_t r, int64_t c, int64_t ld) {
            return (uint64_t)(t ? (c - 1) * ld + r : (r - 1) * ld + c);
        };
        // offset + extent <= size, written so that no sum can wrap around
        auto fits = [](uint64_t off, uint64_t e, uint64_t size) { return e <= size && off <= size - e; };
        if (!fits(seq->a0[i], ext(false, m0, k0, seq->lda0[i]), psi_size) ||
            !fits(seq->b0[i], ext(seq->tb0[i], k0, n0, seq->ldb0[i]), ops_size) ||
            !fits(seq->a1[i], ext(seq->ta1[i], m1, k1, seq->lda1[i]), ops_size) ||
            !fits(seq->c1[i], ext(false, m1, n1, seq->ldc1[i]), sigma_size))
            return fail(B2G_ERR_ARG, "b2g_heff_apply_noalloc: pair " + std::to_string(i) +
                                         " reads or writes out of range");
        if ((uint64_t)(m0 * n0) > kWorkDoubles)
            return fail(B2G_ERR_ARG, "b2g_heff_apply_noalloc: pair " + std::to_string(i) +
                                         " needs a work matrix larger than the " +
                                         std::to_string(kNoAllocScratchBytes >> 20) +
                                         " MiB scratch array");
    }
    int dev = 0;
    B2G_CUDA_TRY(cudaGetDevice(&dev));
    unsigned char *scratch = nullptr;
    int rc = scratch_address(dev, &scratch);
    if (rc != B2G_OK)
        return rc;
    NaPair *d_desc = (NaPair *)scratch;
    double *d_work = (double *)(scratch + kDescBytes);
    cudaStream_t s = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lk(g_mu);  // the host staging array is shared too
    int64_t i = 0;
    while (i < seq->n_pairs) {
        int n = 0;
        uint64_t wused = 0;
        for (; i < seq->n_pairs && n < kChunkPairs; i++) {
            if (seq->m1[i] == 0 || seq->n1[i] == 0 || seq->k1[i] == 0 || seq->k0[i] == 0)
                continue;
            const uint64_t wsz = (uint64_t)seq->m0[i] * seq->n0[i];
            if (wused + wsz > kWorkDoubles)
                break;
            NaPair &p = g_host_desc[n++];
            p.a0 = seq->a0[i], p.b0 = seq->b0[i], p.a1 = seq->a1[i], p.c1 = seq->c1[i];
            p.woff = wused;
            p.alpha0 = seq->alpha0[i], p.alpha1 = seq->alpha1[i];
            p.m0 = seq->m0[i], p.n0 = seq->n0[i], p.k0 = seq->k0[i];
            p.lda0 = seq->lda0[i], p.ldb0 = seq->ldb0[i], p.tb0 = seq->tb0[i] ? 1 : 0;
            p.m1 = seq->m1[i], p.n1 = seq->n1[i], p.k1 = seq->k1[i];
            p.lda1 = seq->lda1[i], p.ldc1 = seq->ldc1[i], p.ta1 = seq->ta1[i] ? 1 : 0;
            wused += wsz;
        }
        if (n == 0)
            continue;
        // pageable source: the call returns once the data is staged, so the
        // host array may be refilled for the next chunk
        B2G_CUDA_TRY(cudaMemcpyAsync(d_desc, g_host_desc, sizeof(NaPair) * n, cudaMemcpyHostToDevice, s));
        note_launch();
        na_gemm0<<<n, 128, 0, s>>>(d_desc, ops, psi, d_work);
        B2G_CUDA_TRY(cudaGetLastError());
        note_launch();
        na_gemm1<<<n, 128, 0, s>>>(d_desc, ops, d_work, sigma, scale);
        B2G_CUDA_TRY(cudaGetLastError());
    }
    return B2G_OK;
}
