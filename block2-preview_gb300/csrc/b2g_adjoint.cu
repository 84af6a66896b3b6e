// The differentiation form: the adjoint of H_eff*psi.
//
// For bra x and ket y the recorded pairs give
//
//   f(ops, y) = <x| H_eff(ops) |y> = sum_p c_p tr(x_p^T A'_p y_p B'_p),
//   c_p = alpha0_p alpha1_p,  A'_p = op_a1(ops[a1:]) (m1 x k1),
//   B'_p = op_b0(ops[b0:]) (k0 x n0),  y_p = y[a0:] (m0 x k0),  x_p = x[c1:] (m1 x n1),
//
// (the pair semantics of BatchGEMMSeq::rotate, src/core/batch_gemm.hpp:893-902,
// through AdvancedGEMM::rotate, batch_gemm.hpp:564-575: work = a op(ket),
// c += scale op(bra) work), so, with W'_p = y_p B'_p and T_p = A'_p^T x_p,
//
//   df/dA'_p = c_p x_p W'_p^T,   df/dB'_p = c_p y_p^T T_p,   df/dy_p = c_p T_p B'_p^T.
//
// The last is (H_eff^T x) restricted to block p.  The operator gradient is a
// list of small dense products C += coef op(A) op(B); three launches of one
// FP64 kernel compute the distinct W' (GEMM0 products, de-duplicated as in
// the forward plan), the distinct T, then the operator gradient.
// Destinations that overlap in memory form one group, processed in a fixed
// order by one CTA (large groups are first cut into disjoint destination
// tiles): deterministic, no atomics.  The ket gradient H_eff^T x is itself a
// forward product, of the transposed pairs
//   W'' = x_p op_b0(B)^T (m1 x k0),  grad_y[a0:] += c_p op_a1(A)^T W''
// (GEMM0 reads x at c1, GEMM1 writes at a0, both operator flags flipped), so
// it runs on the forward FP64 plan and kernels (simt_phase1/2: de-duplicated
// GEMM0, owner-computes sigma regions, deterministic split-K).
#include <algorithm>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "b2g_internal.h"

namespace b2g {

enum { kSrcOps = 0, kSrcY = 1, kSrcX = 2, kSrcW = 3, kSrcT = 4, kNumSrc = 5 };

// C[i][j] (ld ldc) += scale * coef * sum_k opA[i][k] opB[k][j];
// opA[i][k] = ta ? A[k lda + i] : A[i lda + k], opB[k][j] = tb ? B[j ldb + k] : B[k ldb + j]
// restricted to rows [i0, i1) and columns [j0, j1) of C (a group split into
// destination tiles gives each tile its own restricted copy of an item)
struct AdjItem {
    uint64_t a, b, c;
    double coef;
    int32_t M, N, K;
    int32_t lda, ldb, ldc;
    int8_t ta, tb, asrc, bsrc;
    int32_t i0, i1, j0, j1;
};

struct AdjStage {
    AdjItem *items = nullptr;
    int64_t *grp = nullptr;   // items of group g: [grp[g], grp[g + 1])
    int64_t n_items = 0, n_groups = 0;
};

struct AdjointPlan {
    AdjStage st[3];           // W', T, operator gradient
    double *wbuf = nullptr, *tbuf = nullptr;
    uint64_t wsize = 0, tsize = 0;
    uint64_t ops_size = 0, psi_size = 0, sigma_size = 0;
    double mnk = 0;           // multiply-adds of one adjoint (both gradients)
    // ket gradient H_eff^T x: the forward FP64 engine on the transposed pairs
    DevicePlan tplan;
    double *twork = nullptr, *tpart = nullptr;
    uint64_t twork_size = 0, tpart_size = 0;
};

struct AdjSrc {
    const double *p[kNumSrc];
};

constexpr int kAT = 32;       // output tile kAT x kAT, K chunk kAT; 256 threads, 4 cells each

__global__ void __launch_bounds__(256) adj_items(const AdjItem *__restrict__ items,
                                                 const int64_t *__restrict__ grp, int64_t n_groups,
                                                 AdjSrc src, double *__restrict__ dst, double scale) {
    __shared__ double As[kAT][kAT + 1];   // As[k][i]
    __shared__ double Bs[kAT][kAT + 4];   // Bs[k][j]
    const int tid = threadIdx.x;
    const int ti = tid >> 3, tj = (tid & 7) * 4;
    for (int64_t g = blockIdx.x; g < n_groups; g += gridDim.x) {
        for (int64_t it = grp[g]; it < grp[g + 1]; it++) {
            const AdjItem e = items[it];
            const double *__restrict__ A = src.p[e.asrc] + e.a;
            const double *__restrict__ B = src.p[e.bsrc] + e.b;
            const double f = scale * e.coef;
            for (int i0 = e.i0; i0 < e.i1; i0 += kAT) {
                for (int j0 = e.j0; j0 < e.j1; j0 += kAT) {
                    double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0, acc3 = 0.0;
                    for (int k0 = 0; k0 < e.K; k0 += kAT) {
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            // consecutive threads walk the stored matrices' contiguous index
                            const int el = tid + 256 * q, r = el >> 5, c = el & 31;
                            {
                                const int i = e.ta ? c : r, k = e.ta ? r : c;
                                const int gi = i0 + i, gk = k0 + k;
                                double v = 0.0;
                                if (gi < e.i1 && gk < e.K)
                                    v = e.ta ? A[(size_t)gk * e.lda + gi] : A[(size_t)gi * e.lda + gk];
                                As[k][i] = v;
                            }
                            {
                                const int j = e.tb ? r : c, k = e.tb ? c : r;
                                const int gj = j0 + j, gk = k0 + k;
                                double v = 0.0;
                                if (gj < e.j1 && gk < e.K)
                                    v = e.tb ? B[(size_t)gj * e.ldb + gk] : B[(size_t)gk * e.ldb + gj];
                                Bs[k][j] = v;
                            }
                        }
                        __syncthreads();
                        // a warp owns rows [4 w, 4 w + 4) of the tile: warps past the
                        // item's last row skip the products (warp-uniform)
                        const int kn = (i0 + (ti & ~3) < e.i1) ? min(kAT, e.K - k0) : 0;
                        for (int k = 0; k < kn; k++) {
                            const double a = As[k][ti];
                            acc0 = fma(a, Bs[k][tj], acc0);
                            acc1 = fma(a, Bs[k][tj + 1], acc1);
                            acc2 = fma(a, Bs[k][tj + 2], acc2);
                            acc3 = fma(a, Bs[k][tj + 3], acc3);
                        }
                        __syncthreads();
                    }
                    const int gi = i0 + ti;
                    if (gi < e.i1) {
                        double *row = dst + e.c + (size_t)gi * e.ldc;
                        const int gj = j0 + tj;
                        if (gj < e.j1) row[gj] += f * acc0;
                        if (gj + 1 < e.j1) row[gj + 1] += f * acc1;
                        if (gj + 2 < e.j1) row[gj + 2] += f * acc2;
                        if (gj + 3 < e.j1) row[gj + 3] += f * acc3;
                    }
                    // the next tile or item of this group may touch these cells:
                    // the barrier orders this CTA's global writes before its next reads
                    __syncthreads();
                }
            }
        }
    }
}

namespace {

struct HostStage {
    std::vector<AdjItem> items;
    std::vector<int64_t> grp;
};

// stored extent of an operand: rows x cols with leading dimension ld at offset off
bool fits(uint64_t off, int64_t rows, int64_t cols, int64_t ld, uint64_t size) {
    if (rows <= 0 || cols <= 0 || ld < cols)
        return false;
    const uint64_t last = off + (uint64_t)(rows - 1) * (uint64_t)ld + (uint64_t)cols;
    return last <= size && last > off;
}

bool item_ok(const AdjItem &e, const uint64_t *src_size, uint64_t dst_size) {
    if (e.M <= 0 || e.N <= 0 || e.K <= 0 || e.i0 < 0 || e.i1 > e.M || e.i0 >= e.i1 || e.j0 < 0 ||
        e.j1 > e.N || e.j0 >= e.j1)
        return false;
    const bool a = e.ta ? fits(e.a, e.K, e.M, e.lda, src_size[e.asrc]) : fits(e.a, e.M, e.K, e.lda, src_size[e.asrc]);
    const bool b = e.tb ? fits(e.b, e.N, e.K, e.ldb, src_size[e.bsrc]) : fits(e.b, e.K, e.N, e.ldb, src_size[e.bsrc]);
    return a && b && fits(e.c, e.M, e.N, e.ldc, dst_size);
}

// one group per item (destinations owned by a single item)
void single_groups(HostStage &s) {
    s.grp.resize(s.items.size() + 1);
    for (size_t i = 0; i <= s.items.size(); i++)
        s.grp[i] = (int64_t)i;
}

double item_mnk(const AdjItem &e) { return (double)(e.i1 - e.i0) * (e.j1 - e.j0) * e.K; }

// Items whose destination spans overlap share a group; a group keeps its
// items in their original order, groups are ordered by address.  A group
// holding more than max_mnk multiply-adds whose items all write rows of one
// frame (same leading dimension, every item inside the frame's columns) is
// split into kAT x kAT tiles of that frame: one group per tile, holding each
// item restricted to the tile, so no single CTA serialises a large block.
void overlap_groups(HostStage &s, double max_mnk) {
    const size_t n = s.items.size();
    std::vector<uint64_t> lo(n), hi(n);
    std::vector<size_t> ord(n);
    for (size_t i = 0; i < n; i++) {
        const AdjItem &e = s.items[i];
        lo[i] = e.c;
        hi[i] = e.c + (uint64_t)(e.M - 1) * (uint64_t)e.ldc + (uint64_t)e.N;
        ord[i] = i;
    }
    std::stable_sort(ord.begin(), ord.end(), [&](size_t x, size_t y) { return lo[x] < lo[y]; });
    std::vector<AdjItem> out;
    out.reserve(n);
    s.grp.assign(1, 0);
    size_t i = 0;
    while (i < n) {
        size_t j = i + 1;
        uint64_t end = hi[ord[i]];
        while (j < n && lo[ord[j]] < end) {
            end = std::max(end, hi[ord[j]]);
            j++;
        }
        std::vector<size_t> g(ord.begin() + (ptrdiff_t)i, ord.begin() + (ptrdiff_t)j);
        std::sort(g.begin(), g.end());
        double work = 0;
        bool frame = true;
        const int32_t ld = s.items[g[0]].ldc;
        for (size_t k : g) {
            work += item_mnk(s.items[k]);
            frame = frame && s.items[k].ldc == ld;
        }
        // the frame's row start: the lowest item need not start a row, so try
        // the shifts that put some item's first column at column 0
        uint64_t base = lo[ord[i]];
        if (frame && work > max_mnk && g.size() >= 2) {
            std::vector<uint64_t> shifts(1, 0);
            for (size_t k : g)
                shifts.push_back(((uint64_t)ld - (s.items[k].c - base) % (uint64_t)ld) % (uint64_t)ld);
            std::sort(shifts.begin(), shifts.end());
            shifts.erase(std::unique(shifts.begin(), shifts.end()), shifts.end());
            frame = false;
            for (uint64_t sh : shifts) {
                if (sh > base)
                    continue;
                bool ok = true;
                for (size_t k : g)
                    if ((s.items[k].c - (base - sh)) % (uint64_t)ld + (uint64_t)s.items[k].N > (uint64_t)ld) {
                        ok = false;
                        break;
                    }
                if (ok) {
                    base -= sh;
                    frame = true;
                    break;
                }
            }
        }
        if (!frame || work <= max_mnk || g.size() < 2) {
            for (size_t k : g)
                out.push_back(s.items[k]);
            s.grp.push_back((int64_t)out.size());
        } else {
            // frame tile (row band, column band) -> restricted items, in item order
            std::map<std::pair<int64_t, int64_t>, std::vector<AdjItem>> tiles;
            for (size_t k : g) {
                const AdjItem &e = s.items[k];
                const int64_t r0 = (int64_t)((e.c - base) / (uint64_t)ld);
                const int64_t c0 = (int64_t)((e.c - base) % (uint64_t)ld);
                for (int64_t tr = (r0 + e.i0) / kAT; tr * kAT < r0 + e.i1; tr++)
                    for (int64_t tc = (c0 + e.j0) / kAT; tc * kAT < c0 + e.j1; tc++) {
                        AdjItem t = e;
                        t.i0 = (int32_t)std::max<int64_t>(e.i0, tr * kAT - r0);
                        t.i1 = (int32_t)std::min<int64_t>(e.i1, (tr + 1) * kAT - r0);
                        t.j0 = (int32_t)std::max<int64_t>(e.j0, tc * kAT - c0);
                        t.j1 = (int32_t)std::min<int64_t>(e.j1, (tc + 1) * kAT - c0);
                        if (t.i0 < t.i1 && t.j0 < t.j1)
                            tiles[std::make_pair(tr, tc)].push_back(t);
                    }
            }
            for (auto &kv : tiles) {
                out.insert(out.end(), kv.second.begin(), kv.second.end());
                s.grp.push_back((int64_t)out.size());
            }
        }
        i = j;
    }
    s.items.swap(out);
}

int upload_stage(const HostStage &h, AdjStage &d, cudaStream_t s) {
    d.n_items = (int64_t)h.items.size();
    d.n_groups = (int64_t)h.grp.size() - 1;
    if (d.n_items == 0)
        return B2G_OK;
    if (cudaMalloc(&d.items, sizeof(AdjItem) * h.items.size()) != cudaSuccess ||
        cudaMalloc(&d.grp, sizeof(int64_t) * h.grp.size()) != cudaSuccess)
        return fail(B2G_ERR_NOMEM, "cudaMalloc failed for the adjoint plan");
    B2G_CUDA_TRY(cudaMemcpyAsync(d.items, h.items.data(), sizeof(AdjItem) * h.items.size(),
                                 cudaMemcpyHostToDevice, s));
    B2G_CUDA_TRY(cudaMemcpyAsync(d.grp, h.grp.data(), sizeof(int64_t) * h.grp.size(),
                                 cudaMemcpyHostToDevice, s));
    return B2G_OK;
}

template <typename T> int upload_vec(const std::vector<T> &v, T **dst, cudaStream_t s) {
    *dst = nullptr;
    if (v.empty())
        return B2G_OK;
    if (cudaMalloc((void **)dst, sizeof(T) * v.size()) != cudaSuccess) {
        *dst = nullptr;
        return fail(B2G_ERR_NOMEM, "cudaMalloc failed for the adjoint's transposed plan");
    }
    B2G_CUDA_TRY(cudaMemcpyAsync(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, s));
    return B2G_OK;
}

// the FP64 (CUDA-core) tables of a forward plan
int upload_simt_plan(const HostPlan &hp, DevicePlan &p, cudaStream_t s) {
    int rc;
    if ((rc = upload_vec(hp.works, &p.works, s)) || (rc = upload_vec(hp.contribs, &p.contribs, s)) ||
        (rc = upload_vec(hp.regions, &p.regions, s)) || (rc = upload_vec(hp.t1, &p.t1, s)) ||
        (rc = upload_vec(hp.t2, &p.t2, s)) || (rc = upload_vec(hp.lists, &p.lists, s)) ||
        (rc = upload_vec(hp.t2multi, &p.t2multi, s)))
        return rc;
    p.n_works = (int64_t)hp.works.size(), p.n_contribs = (int64_t)hp.contribs.size();
    p.n_regions = (int64_t)hp.regions.size(), p.n_t1 = (int64_t)hp.t1.size();
    p.n_t2 = (int64_t)hp.t2.size(), p.n_lists = (int64_t)hp.lists.size();
    p.n_t2multi = (int64_t)hp.t2multi.size();
    return B2G_OK;
}

cudaError_t launch_stage(const AdjStage &st, const AdjSrc &src, double *dst, double scale,
                         cudaStream_t s) {
    if (st.n_groups == 0)
        return cudaSuccess;
    const int64_t grid = std::min<int64_t>(st.n_groups, (int64_t)1 << 20);
    note_launch();
    adj_items<<<(unsigned)grid, 256, 0, s>>>(st.items, st.grp, st.n_groups, src, dst, scale);
    return cudaGetLastError();
}

} // namespace

void free_adjoint(b2g_heff *h) {
    AdjointPlan *p = h->adj;
    if (p == nullptr)
        return;
    for (AdjStage &s : p->st)
        cudaFree(s.items), cudaFree(s.grp);
    cudaFree(p->wbuf), cudaFree(p->tbuf);
    DevicePlan &t = p->tplan;
    cudaFree(t.works), cudaFree(t.contribs), cudaFree(t.regions), cudaFree(t.t1), cudaFree(t.t2);
    cudaFree(t.lists), cudaFree(t.t2multi);
    cudaFree(p->twork), cudaFree(p->tpart);
    delete p;
    h->adj = nullptr;
}

} // namespace b2g

using namespace b2g;

extern "C" {

int b2g_heff_set_ops(b2g_heff *h, const double *ops, int ops_on_device) {
    if (h == nullptr || (ops == nullptr && h->ops_size != 0))
        return fail(B2G_ERR_ARG, "b2g_heff_set_ops: null argument");
    if (h->ops_size == 0)
        return B2G_OK;
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    cudaStream_t s = h->ctx->stream;
    B2G_CUDA_TRY(cudaMemcpyAsync(h->ops, ops, sizeof(double) * h->ops_size,
                                 ops_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
    // the reduced-precision copies made from the blob follow it (same buffers,
    // so captured applies stay valid)
    if (h->ops32 != nullptr)
        B2G_CUDA_TRY(launch_to_float(h->ops, h->ops32, h->ops_size, s));
    if (h->g1_aimg != nullptr && h->ops32 != nullptr)
        B2G_CUDA_TRY(launch_g1_build_a(h->plan, h->ops32, h->g1_aimg, s));
    if (!ops_on_device)
        B2G_CUDA_TRY(cudaStreamSynchronize(s));
    return B2G_OK;
}

int b2g_heff_adjoint_prepare(b2g_heff *h, const b2g_pair_seq *seq) {
    if (h == nullptr || seq == nullptr || seq->n_pairs < 0)
        return fail(B2G_ERR_ARG, "b2g_heff_adjoint_prepare: null argument");
    if (seq->n_pairs != h->stats.n_pairs)
        return fail(B2G_ERR_ARG, "b2g_heff_adjoint_prepare: the sequence is not the one the H_eff was built from");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    cudaStream_t s = h->ctx->stream;
    B2G_CUDA_TRY(cudaStreamSynchronize(s));
    free_adjoint(h);
    const int64_t n = seq->n_pairs;
    HostStage hw, ht, hg;
    std::map<std::tuple<uint64_t, uint64_t, int, int, int, int, int, int>, uint64_t> wkey;
    std::map<std::tuple<uint64_t, uint64_t, int, int, int, int, int, int>, uint64_t> tkey;
    uint64_t wsize = 0, tsize = 0;
    double mnk = 0;
    std::vector<uint64_t> woff(n), toff(n);
    for (int64_t p = 0; p < n; p++) {
        const int m0 = seq->m0[p], n0 = seq->n0[p], k0 = seq->k0[p];
        const int m1 = seq->m1[p], n1 = seq->n1[p], k1 = seq->k1[p];
        if (k1 != m0 || n1 != n0)
            return fail(B2G_ERR_ARG, "b2g_heff_adjoint_prepare: pair " + std::to_string(p) +
                                         " has k1 != m0 or n1 != n0");
        auto kw = std::make_tuple(seq->a0[p], seq->b0[p], seq->tb0[p], m0, n0, k0, seq->lda0[p], seq->ldb0[p]);
        auto iw = wkey.find(kw);
        if (iw == wkey.end()) {
            iw = wkey.emplace(kw, wsize).first;
            AdjItem e{};
            e.a = seq->a0[p], e.b = seq->b0[p], e.c = wsize, e.coef = 1.0;
            e.M = m0, e.N = n0, e.K = k0, e.lda = seq->lda0[p], e.ldb = seq->ldb0[p], e.ldc = n0;
            e.ta = 0, e.tb = seq->tb0[p] ? 1 : 0, e.asrc = kSrcY, e.bsrc = kSrcOps;
            e.i0 = 0, e.i1 = e.M, e.j0 = 0, e.j1 = e.N;
            hw.items.push_back(e);
            wsize += (uint64_t)m0 * n0;
            mnk += (double)m0 * n0 * k0;
        }
        woff[p] = iw->second;
        auto kt = std::make_tuple(seq->a1[p], seq->c1[p], seq->ta1[p], m1, k1, n1, seq->lda1[p], seq->ldc1[p]);
        auto itt = tkey.find(kt);
        if (itt == tkey.end()) {
            itt = tkey.emplace(kt, tsize).first;
            AdjItem e{};   // T = op_a1(A)^T x_p  (k1 x n1)
            e.a = seq->a1[p], e.b = seq->c1[p], e.c = tsize, e.coef = 1.0;
            e.M = k1, e.N = n1, e.K = m1, e.lda = seq->lda1[p], e.ldb = seq->ldc1[p], e.ldc = n1;
            e.ta = seq->ta1[p] ? 0 : 1, e.tb = 0, e.asrc = kSrcOps, e.bsrc = kSrcX;
            e.i0 = 0, e.i1 = e.M, e.j0 = 0, e.j1 = e.N;
            ht.items.push_back(e);
            tsize += (uint64_t)k1 * n1;
            mnk += (double)k1 * n1 * m1;
        }
        toff[p] = itt->second;
        const double coef = seq->alpha0[p] * seq->alpha1[p];
        AdjItem a{};   // operator gradient of the GEMM1 (bra-side) block
        a.coef = coef, a.c = seq->a1[p], a.ldc = seq->lda1[p];
        if (!seq->ta1[p]) {   // dA (m1 x k1) = x_p W'^T
            a.M = m1, a.N = k1, a.K = n1;
            a.a = seq->c1[p], a.lda = seq->ldc1[p], a.ta = 0, a.asrc = kSrcX;
            a.b = woff[p], a.ldb = n0, a.tb = 1, a.bsrc = kSrcW;
        } else {              // dA (k1 x m1) = W' x_p^T
            a.M = k1, a.N = m1, a.K = n0;
            a.a = woff[p], a.lda = n0, a.ta = 0, a.asrc = kSrcW;
            a.b = seq->c1[p], a.ldb = seq->ldc1[p], a.tb = 1, a.bsrc = kSrcX;
        }
        a.i0 = 0, a.i1 = a.M, a.j0 = 0, a.j1 = a.N;
        hg.items.push_back(a);
        AdjItem b{};   // operator gradient of the GEMM0 (ket-side) block
        b.coef = coef, b.c = seq->b0[p], b.ldc = seq->ldb0[p];
        if (!seq->tb0[p]) {   // dB (k0 x n0) = y_p^T T
            b.M = k0, b.N = n0, b.K = m0;
            b.a = seq->a0[p], b.lda = seq->lda0[p], b.ta = 1, b.asrc = kSrcY;
            b.b = toff[p], b.ldb = n0, b.tb = 0, b.bsrc = kSrcT;
        } else {              // dB (n0 x k0) = T^T y_p
            b.M = n0, b.N = k0, b.K = m0;
            b.a = toff[p], b.lda = n0, b.ta = 1, b.asrc = kSrcT;
            b.b = seq->a0[p], b.ldb = seq->lda0[p], b.tb = 0, b.bsrc = kSrcY;
        }
        b.i0 = 0, b.i1 = b.M, b.j0 = 0, b.j1 = b.N;
        hg.items.push_back(b);
        mnk += (double)m1 * k1 * n1 + (double)k0 * n0 * m0;
    }
    // the transposed pairs (ket gradient = forward product of these with psi := x)
    std::vector<int32_t> t_tb0(n), t_m0(n), t_n0(n), t_k0(n), t_lda0(n), t_ldb0(n);
    std::vector<int32_t> t_ta1(n), t_m1(n), t_n1(n), t_k1(n), t_lda1(n), t_ldc1(n);
    std::vector<double> t_al0(n), t_al1(n);
    std::vector<uint64_t> t_a0(n), t_b0(n), t_a1(n), t_c1(n);
    for (int64_t p = 0; p < n; p++) {
        t_tb0[p] = seq->tb0[p] ? 0 : 1, t_m0[p] = seq->m1[p], t_k0[p] = seq->n1[p], t_n0[p] = seq->k0[p];
        t_lda0[p] = seq->ldc1[p], t_ldb0[p] = seq->ldb0[p], t_a0[p] = seq->c1[p], t_b0[p] = seq->b0[p];
        t_ta1[p] = seq->ta1[p] ? 0 : 1, t_m1[p] = seq->m0[p], t_k1[p] = seq->m1[p], t_n1[p] = seq->k0[p];
        t_lda1[p] = seq->lda1[p], t_ldc1[p] = seq->lda0[p], t_a1[p] = seq->a1[p], t_c1[p] = seq->a0[p];
        t_al0[p] = seq->alpha0[p], t_al1[p] = seq->alpha1[p];
    }
    b2g_pair_seq tseq;
    tseq.n_pairs = n;
    tseq.tb0 = t_tb0.data(), tseq.m0 = t_m0.data(), tseq.n0 = t_n0.data(), tseq.k0 = t_k0.data();
    tseq.lda0 = t_lda0.data(), tseq.ldb0 = t_ldb0.data(), tseq.ta1 = t_ta1.data(), tseq.m1 = t_m1.data();
    tseq.n1 = t_n1.data(), tseq.k1 = t_k1.data(), tseq.lda1 = t_lda1.data(), tseq.ldc1 = t_ldc1.data();
    tseq.alpha0 = t_al0.data(), tseq.alpha1 = t_al1.data();
    tseq.a0 = t_a0.data(), tseq.b0 = t_b0.data(), tseq.a1 = t_a1.data(), tseq.c1 = t_c1.data();
    HostPlan thp;
    int trc = build_plan(&tseq, h->ops_size, h->sigma_size, h->psi_size, thp);
    if (trc != B2G_OK)
        return trc;
    mnk += thp.mnk_exec;
    // every operand of every item inside its buffer (nothing reaches the GPU unchecked)
    const uint64_t sizes[kNumSrc] = {h->ops_size, h->psi_size, h->sigma_size, wsize, tsize};
    const struct { const HostStage *s; uint64_t dst; const char *name; } checks[3] = {
        {&hw, wsize, "W"}, {&ht, tsize, "T"}, {&hg, h->ops_size, "operator gradient"}};
    for (const auto &c : checks)
        for (size_t i = 0; i < c.s->items.size(); i++)
            if (!item_ok(c.s->items[i], sizes, c.dst))
                return fail(B2G_ERR_ARG, std::string("b2g_heff_adjoint_prepare: a ") + c.name +
                                             " product reaches outside its buffers (pair sizes or offsets)");
    single_groups(hw);
    single_groups(ht);
    // no group above 1/4096 of a stage's work (2 CTAs on each of 152 SMs,
    // about 13 groups each) unless its items cannot be tiled
    double wg = 0;
    for (const AdjItem &e : hg.items)
        wg += item_mnk(e);
    overlap_groups(hg, wg / 4096.0);
    AdjointPlan *ap = new AdjointPlan();
    h->adj = ap;
    ap->wsize = wsize, ap->tsize = tsize, ap->mnk = mnk;
    ap->ops_size = h->ops_size, ap->psi_size = h->psi_size, ap->sigma_size = h->sigma_size;
    int rc;
    if ((rc = upload_stage(hw, ap->st[0], s)) || (rc = upload_stage(ht, ap->st[1], s)) ||
        (rc = upload_stage(hg, ap->st[2], s)) || (rc = upload_simt_plan(thp, ap->tplan, s))) {
        free_adjoint(h);
        return rc;
    }
    ap->twork_size = thp.work_size;
    ap->tpart_size = (uint64_t)4 * 256 * thp.t2_part_tiles;
    if ((wsize && cudaMalloc(&ap->wbuf, sizeof(double) * wsize) != cudaSuccess) ||
        (tsize && cudaMalloc(&ap->tbuf, sizeof(double) * tsize) != cudaSuccess) ||
        (ap->twork_size && cudaMalloc(&ap->twork, sizeof(double) * ap->twork_size) != cudaSuccess) ||
        (ap->tpart_size && cudaMalloc(&ap->tpart, sizeof(double) * ap->tpart_size) != cudaSuccess)) {
        free_adjoint(h);
        return fail(B2G_ERR_NOMEM, "cudaMalloc failed for the adjoint work matrices");
    }
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        free_adjoint(h);
        return fail(B2G_ERR_CUDA, "adjoint plan upload failed");
    }
    return B2G_OK;
}

int b2g_heff_adjoint(b2g_heff *h, const double *x, const double *y, double scale, double *grad_ops,
                     double *grad_psi) {
    if (h == nullptr || (grad_ops == nullptr && grad_psi == nullptr))
        return fail(B2G_ERR_ARG, "b2g_heff_adjoint: null argument");
    if (h->adj == nullptr)
        return fail(B2G_ERR_STATE, "b2g_heff_adjoint: call b2g_heff_adjoint_prepare first");
    if ((h->sigma_size && x == nullptr) || (grad_ops != nullptr && h->psi_size && y == nullptr))
        return fail(B2G_ERR_ARG, "b2g_heff_adjoint: null bra or ket");
    B2G_CUDA_TRY(cudaSetDevice(h->ctx->device));
    const AdjointPlan &p = *h->adj;
    cudaStream_t s = h->ctx->stream;
    AdjSrc src{{h->ops, y, x, p.wbuf, p.tbuf}};
    if (grad_ops != nullptr) {
        if (p.tsize) {
            B2G_CUDA_TRY(cudaMemsetAsync(p.tbuf, 0, sizeof(double) * p.tsize, s));
            B2G_CUDA_TRY(launch_stage(p.st[1], src, p.tbuf, 1.0, s));
        }
        if (p.wsize) {
            B2G_CUDA_TRY(cudaMemsetAsync(p.wbuf, 0, sizeof(double) * p.wsize, s));
            B2G_CUDA_TRY(launch_stage(p.st[0], src, p.wbuf, 1.0, s));
        }
        B2G_CUDA_TRY(launch_stage(p.st[2], src, grad_ops, scale, s));
    }
    if (grad_psi != nullptr) {
        RootStrides rs;
        rs.nroots = 1, rs.psi = p.sigma_size, rs.sigma = p.psi_size;
        rs.work = p.twork_size, rs.part = p.tpart_size;
        B2G_CUDA_TRY(launch_simt_phase1<double>(p.tplan, h->ops, x, p.twork, rs, s));
        B2G_CUDA_TRY(launch_simt_phase2<double>(p.tplan, h->ops, p.twork, grad_psi, p.tpart, scale, rs, s));
    }
    return B2G_OK;
}

int b2g_heff_adjoint_mnk(const b2g_heff *h, double *mnk) {
    if (h == nullptr || mnk == nullptr)
        return fail(B2G_ERR_ARG, "b2g_heff_adjoint_mnk: null argument");
    if (h->adj == nullptr)
        return fail(B2G_ERR_STATE, "b2g_heff_adjoint_mnk: call b2g_heff_adjoint_prepare first");
    *mnk = h->adj->mnk;
    return B2G_OK;
}

} // extern "C"
