// Environment blocking (the enlarged block's operators) on the device, FP64.
//
// The reference builds the operators of the enlarged left (right) block in
// TensorFunctions::left_contract / right_contract
// (src/core/tensor_functions.hpp:2842-2986): every new operator is a sum of
// Kronecker products of an environment operator and a site operator, where
// some factors are themselves sums of operators.  At block level that is two
// kinds of records (as the recorder of the reference logs them):
//   iadd  (OperatorFunctions::iadd, src/core/operator_functions.hpp:135-170):
//         tmp[dst](m x n) += f * op(src)            (op = transpose if conj)
//   kron  (OperatorFunctions::tensor_product, operator_functions.hpp:672-710;
//         GMatrixFunctions::tensor_product, src/core/matrix_functions.hpp:1269):
//         out[c + (i bm' + k) cn + j bn' + l] += f * A'(i,j) * B'(k,l)
//         with A' = op(a) (am' x an'), B' = op(b) (bm' x bn').
// Operands come from four blobs: 0 environment operators, 1 site operators,
// 2 intermediates (made by the iadd records), 3 output.  The iadd records run
// first (an intermediate is complete before any product reads it), then the
// kron records.  Records that write overlapping ranges form one group,
// processed by one CTA in recorded order (no atomics, reproducible); groups run
// in parallel.
#include <algorithm>
#include <numeric>
#include <vector>

#include "b2g_internal.h"

namespace b2g {

namespace {

struct BlkIadd {
    uint64_t dst, src;
    double f;
    int32_t m, n, conj, src_blob;
};
struct BlkKron {
    uint64_t a, b, c;
    double f;
    int32_t am, an, bm, bn, ca, cb, cn, ablob, bblob, pad;
};

__device__ __forceinline__ const double *blob_ptr(int id, const double *env, const double *site,
                                                  const double *tmp) {
    return id == 0 ? env : id == 1 ? site : tmp;
}

__global__ void __launch_bounds__(256) iadd_kernel(const BlkIadd *__restrict__ recs,
                                                   const int64_t *__restrict__ grp,
                                                   const double *__restrict__ env,
                                                   const double *__restrict__ site,
                                                   double *__restrict__ tmp) {
    for (int64_t q = grp[blockIdx.x]; q < grp[blockIdx.x + 1]; q++) {
        const BlkIadd r = recs[q];
        const double *src = blob_ptr(r.src_blob, env, site, tmp) + r.src;
        double *dst = tmp + r.dst;
        for (int e = threadIdx.x; e < r.m * r.n; e += blockDim.x) {
            const int i = e / r.n, j = e - i * r.n;
            dst[e] += r.f * (r.conj ? src[(int64_t)j * r.m + i] : src[e]);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) kron_kernel(const BlkKron *__restrict__ recs,
                                                   const int64_t *__restrict__ grp,
                                                   const double *__restrict__ env,
                                                   const double *__restrict__ site,
                                                   const double *__restrict__ tmp,
                                                   double *__restrict__ out) {
    for (int64_t q = grp[blockIdx.x]; q < grp[blockIdx.x + 1]; q++) {
        const BlkKron r = recs[q];
        const double *A = blob_ptr(r.ablob, env, site, tmp) + r.a;
        const double *B = blob_ptr(r.bblob, env, site, tmp) + r.b;
        const int am = r.ca ? r.an : r.am, an = r.ca ? r.am : r.an;  // op(a) dims
        const int bm = r.cb ? r.bn : r.bm, bn = r.cb ? r.bm : r.bn;  // op(b) dims
        const int64_t total = (int64_t)am * an * bm * bn;
        for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
            // e -> (i, k, j, l): output row i bm + k, column j bn + l
            const int l = (int)(e % bn);
            int64_t t = e / bn;
            const int j = (int)(t % an);
            t /= an;
            const int k = (int)(t % bm);
            const int i = (int)(t / bm);
            const double av = r.ca ? A[(int64_t)j * r.an + i] : A[(int64_t)i * r.an + j];
            const double bv = r.cb ? B[(int64_t)l * r.bn + k] : B[(int64_t)k * r.bn + l];
            out[r.c + ((int64_t)i * bm + k) * r.cn + (int64_t)j * bn + l] += r.f * av * bv;
        }
        __syncthreads();
    }
}

// group boundaries of records ordered by their first written element, merging
// records whose written spans overlap; order inside a group stays the recorded one
template <typename Span>
void group_overlapping(int64_t n, Span span, std::vector<int64_t> &order, std::vector<int64_t> &grp) {
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t x, int64_t y) { return span(x).first < span(y).first; });
    grp.clear();
    uint64_t end = 0;
    for (int64_t p = 0; p < n; p++) {
        const auto sp = span(order[p]);
        if (p == 0 || sp.first >= end) {
            grp.push_back(p);
            end = sp.second;
        } else
            end = std::max(end, sp.second);
    }
    grp.push_back(n);
    // recorded order inside each group
    for (size_t g = 0; g + 1 < grp.size(); g++)
        std::sort(order.begin() + grp[g], order.begin() + grp[g + 1]);
}

} // namespace

} // namespace b2g

using namespace b2g;

static int block_contract(b2g_context *ctx, const b2g_block_seq *seq, const double *env,
                          uint64_t env_size, const double *site, uint64_t site_size,
                          uint64_t tmp_size, double *out, uint64_t out_size, bool on_device) {
    if (ctx == nullptr || seq == nullptr || out == nullptr || (env_size && env == nullptr) ||
        (site_size && site == nullptr) || seq->n_iadd < 0 || seq->n_kron < 0)
        return fail(B2G_ERR_ARG, "b2g_block_contract: null or negative argument");
    const uint64_t sizes[3] = {env_size, site_size, tmp_size};
    // ---- records with bounds checks (every read and write stays inside its blob)
    std::vector<BlkIadd> ia((size_t)seq->n_iadd);
    for (int64_t q = 0; q < seq->n_iadd; q++) {
        BlkIadd &r = ia[q];
        r.dst = seq->ia_dst[q], r.src = seq->ia_src[q], r.f = seq->ia_f[q];
        r.m = seq->ia_m[q], r.n = seq->ia_n[q], r.conj = seq->ia_conj[q] ? 1 : 0;
        r.src_blob = seq->ia_src_blob[q];
        const uint64_t cnt = (uint64_t)r.m * (uint64_t)r.n;
        if (r.src_blob == 2)
            return fail(B2G_ERR_UNSUPPORTED, "b2g_block_contract: an intermediate built from an intermediate");
        if (r.m < 0 || r.n < 0 || r.src_blob < 0 || r.src_blob > 2 || r.dst + cnt > tmp_size ||
            r.src + cnt > sizes[r.src_blob])
            return fail(B2G_ERR_ARG, "b2g_block_contract: iadd record " + std::to_string(q) + " out of range");
    }
    std::vector<BlkKron> kr((size_t)seq->n_kron);
    for (int64_t q = 0; q < seq->n_kron; q++) {
        BlkKron &r = kr[q];
        r.a = seq->kr_a[q], r.b = seq->kr_b[q], r.c = seq->kr_c[q], r.f = seq->kr_f[q];
        r.am = seq->kr_am[q], r.an = seq->kr_an[q], r.bm = seq->kr_bm[q], r.bn = seq->kr_bn[q];
        r.ca = seq->kr_ca[q] ? 1 : 0, r.cb = seq->kr_cb[q] ? 1 : 0, r.cn = seq->kr_cn[q];
        r.ablob = seq->kr_ablob[q], r.bblob = seq->kr_bblob[q], r.pad = 0;
        const int am = r.ca ? r.an : r.am, an = r.ca ? r.am : r.an;
        const int bm = r.cb ? r.bn : r.bm, bn = r.cb ? r.bm : r.bn;
        if (r.am < 0 || r.an < 0 || r.bm < 0 || r.bn < 0 || r.ablob < 0 || r.ablob > 2 || r.bblob < 0 ||
            r.bblob > 2 || r.a + (uint64_t)r.am * r.an > sizes[r.ablob] ||
            r.b + (uint64_t)r.bm * r.bn > sizes[r.bblob] || (int64_t)an * bn > r.cn)
            return fail(B2G_ERR_ARG, "b2g_block_contract: kron record " + std::to_string(q) + " out of range");
        if (am > 0 && an > 0 && bm > 0 && bn > 0 &&
            r.c + ((uint64_t)am * bm - 1) * (uint64_t)r.cn + (uint64_t)an * bn > out_size)
            return fail(B2G_ERR_ARG, "b2g_block_contract: kron record " + std::to_string(q) + " writes past the output");
    }
    std::vector<int64_t> ia_order, ia_grp, kr_order, kr_grp;
    group_overlapping((int64_t)ia.size(), [&](int64_t q) {
        return std::make_pair(ia[q].dst, ia[q].dst + (uint64_t)ia[q].m * ia[q].n);
    }, ia_order, ia_grp);
    group_overlapping((int64_t)kr.size(), [&](int64_t q) {
        const BlkKron &r = kr[q];
        const uint64_t rows = (uint64_t)(r.ca ? r.an : r.am) * (r.cb ? r.bn : r.bm);
        const uint64_t cols = (uint64_t)(r.ca ? r.am : r.an) * (r.cb ? r.bm : r.bn);
        return std::make_pair(r.c, rows == 0 || cols == 0 ? r.c : r.c + (rows - 1) * r.cn + cols);
    }, kr_order, kr_grp);
    std::vector<BlkIadd> ia_s(ia.size());
    std::vector<BlkKron> kr_s(kr.size());
    for (size_t p = 0; p < ia.size(); p++)
        ia_s[p] = ia[ia_order[p]];
    for (size_t p = 0; p < kr.size(); p++)
        kr_s[p] = kr[kr_order[p]];
    B2G_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    // device operands: the caller's (on_device) or staged copies of the host
    // buffers; scratch from the stream-ordered pool (no synchronisation)
    double *d_env = on_device ? const_cast<double *>(env) : nullptr;
    double *d_site = on_device ? const_cast<double *>(site) : nullptr;
    double *d_out = on_device ? out : nullptr, *d_tmp = nullptr;
    BlkIadd *d_ia = nullptr;
    BlkKron *d_kr = nullptr;
    int64_t *d_iag = nullptr, *d_krg = nullptr;
    auto cleanup = [&]() {
        if (!on_device) {
            cudaFreeAsync(d_env, s), cudaFreeAsync(d_site, s), cudaFreeAsync(d_out, s);
        }
        cudaFreeAsync(d_tmp, s);
        cudaFreeAsync(d_ia, s), cudaFreeAsync(d_kr, s), cudaFreeAsync(d_iag, s), cudaFreeAsync(d_krg, s);
    };
    auto dmalloc = [&](void **p, size_t bytes) { return cudaMallocAsync(p, std::max<size_t>(bytes, 16), s); };
    if ((!on_device && (dmalloc((void **)&d_env, sizeof(double) * env_size) ||
                        dmalloc((void **)&d_site, sizeof(double) * site_size) ||
                        dmalloc((void **)&d_out, sizeof(double) * out_size))) ||
        dmalloc((void **)&d_tmp, sizeof(double) * tmp_size) ||
        dmalloc((void **)&d_ia, sizeof(BlkIadd) * ia_s.size()) || dmalloc((void **)&d_kr, sizeof(BlkKron) * kr_s.size()) ||
        dmalloc((void **)&d_iag, sizeof(int64_t) * ia_grp.size()) ||
        dmalloc((void **)&d_krg, sizeof(int64_t) * kr_grp.size())) {
        cleanup();
        return fail(B2G_ERR_NOMEM, "b2g_block_contract: device allocation failed");
    }
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t x) {
        if (e == cudaSuccess)
            e = x;
    };
    if (!on_device) {
        step(cudaMemcpyAsync(d_env, env, sizeof(double) * env_size, cudaMemcpyHostToDevice, s));
        step(cudaMemcpyAsync(d_site, site, sizeof(double) * site_size, cudaMemcpyHostToDevice, s));
    }
    step(cudaMemsetAsync(d_tmp, 0, sizeof(double) * std::max<uint64_t>(tmp_size, 1), s));
    if (out_size)
        step(cudaMemsetAsync(d_out, 0, sizeof(double) * out_size, s));
    if (!ia_s.empty()) {
        step(cudaMemcpyAsync(d_ia, ia_s.data(), sizeof(BlkIadd) * ia_s.size(), cudaMemcpyHostToDevice, s));
        step(cudaMemcpyAsync(d_iag, ia_grp.data(), sizeof(int64_t) * ia_grp.size(), cudaMemcpyHostToDevice, s));
        if (e == cudaSuccess) {
            note_launch();
            iadd_kernel<<<(unsigned)(ia_grp.size() - 1), 256, 0, s>>>(d_ia, d_iag, d_env, d_site, d_tmp);
            step(cudaGetLastError());
        }
    }
    if (!kr_s.empty()) {
        step(cudaMemcpyAsync(d_kr, kr_s.data(), sizeof(BlkKron) * kr_s.size(), cudaMemcpyHostToDevice, s));
        step(cudaMemcpyAsync(d_krg, kr_grp.data(), sizeof(int64_t) * kr_grp.size(), cudaMemcpyHostToDevice, s));
        if (e == cudaSuccess) {
            note_launch();
            kron_kernel<<<(unsigned)(kr_grp.size() - 1), 256, 0, s>>>(d_kr, d_krg, d_env, d_site, d_tmp, d_out);
            step(cudaGetLastError());
        }
    }
    if (!on_device && out_size)
        step(cudaMemcpyAsync(out, d_out, sizeof(double) * out_size, cudaMemcpyDeviceToHost, s));
    // the record tables live in host vectors of this call: finish before returning
    step(cudaStreamSynchronize(s));
    cleanup();
    if (e != cudaSuccess)
        return fail(B2G_ERR_CUDA, std::string("b2g_block_contract: ") + cudaGetErrorString(e));
    return B2G_OK;
}

extern "C" int b2g_block_contract(b2g_context *ctx, const b2g_block_seq *seq, const double *env,
                                  uint64_t env_size, const double *site, uint64_t site_size,
                                  uint64_t tmp_size, double *out, uint64_t out_size) {
    return block_contract(ctx, seq, env, env_size, site, site_size, tmp_size, out, out_size, false);
}

extern "C" int b2g_block_contract_device(b2g_context *ctx, const b2g_block_seq *seq, const double *env,
                                         uint64_t env_size, const double *site, uint64_t site_size,
                                         uint64_t tmp_size, double *out, uint64_t out_size) {
    return block_contract(ctx, seq, env, env_size, site, site_size, tmp_size, out, out_size, true);
}
