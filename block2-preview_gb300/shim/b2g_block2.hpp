// b2g_block2.hpp -- the block2 side of the GB300 drop-in (header-only C++).
//
// Included after block2's own headers ("block2_core.hpp", "block2_dmrg.hpp")
// and linked against libb2g.so.  It adds two subclasses that plug into
// block2's virtual hooks, so block2's MovingEnvironment, EffectiveHamiltonian
// and DMRG::solve / sweep run unchanged above the GPU path:
//
//   GpuTensorFunctions<S>  a TensorFunctions<S, double> installed as mpo->tf
//                          (block2 copies it into every EffectiveHamiltonian,
//                          src/dmrg/effective_hamiltonian.hpp:136).  Its
//                          operator()(b, c, scale) -- the product Davidson
//                          calls after EffectiveHamiltonian::precompute has
//                          recorded the GEMM pairs (src/core/tensor_functions.hpp:59-62,
//                          src/dmrg/effective_hamiltonian.hpp:514-532) --
//                          replays the recorded pairs on the GPU instead of
//                          BatchGEMMSeq::operator() (src/core/batch_gemm.hpp:1570-1690);
//                          its tensor_product_partial_multiply runs the
//                          perturbative-noise product (the GEMM list
//                          EffectiveHamiltonian::perturbative_noise records,
//                          src/dmrg/effective_hamiltonian.hpp:262-433) on the GPU.
//   GpuDMRG<S>             a DMRG<S, double, double> whose virtual
//                          two_dot_eigs_and_perturb (src/dmrg/sweep_algorithm.hpp:1183-1268)
//                          runs the whole Davidson solve on the device
//                          (b2g_davidson) in the selected arithmetic form, with
//                          diag(H_eff) computed on the device from the pairs.
//
// Errors: a non-zero status of the C ABI becomes std::runtime_error carrying
// b2g_last_error(), block2's own error convention.  Options this GPU path does
// not implement (metric, state-specific or projected solves, parallel rules,
// non-Normal Davidson types, non-Tasked GEMM sequences) raise instead of
// running on the host.
#pragma once

#include "b2g.h"

#include <algorithm>
#include <atomic>
#include <fstream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

namespace b2g_block2 {

inline void check(int rc, const char *what) {
    if (rc != B2G_OK)
        throw std::runtime_error(std::string(what) + ": " + b2g_last_error());
}

// One device context shared by every copy of the tensor functions.
struct Runtime {
    b2g_context *ctx = nullptr;
    int form = B2G_FP64;        // arithmetic of the Davidson expansion products
    // counters over the run (read by the driver program)
    long long n_heff = 0, n_apply_fp64 = 0, n_apply_reduced = 0;
    double t_plan = 0, t_upload = 0;
    double t_davidson = 0;      // wall time inside b2g_davidson (device-resident solves)
    double h2d_bytes = 0, d2h_bytes = 0;  // host<->device traffic of the drop-in
    // perturbative noise (EffectiveHamiltonian::perturbative_noise) on the device;
    // false: block2 replays its recorded GEMM list on the host
    bool noise_on_device = true;
    long long n_noise = 0;
    long long n_expect = 0;  // fast-expectation products (PDM sweeps) run on the device
    std::atomic<int> noise_depth{0};  // nesting of tensor_product_partial_multiply
    explicit Runtime(int device = 0, int form = B2G_FP64) : form(form) {
        check(b2g_context_create(device, &ctx), "b2g_context_create");
    }
    ~Runtime() {
        if (ctx != nullptr)
            b2g_context_destroy(ctx);
    }
    Runtime(const Runtime &) = delete;
    Runtime &operator=(const Runtime &) = delete;
};

// The GEMM pairs block2 recorded for one H_eff*psi, translated into the C
// ABI's pair format: psi / sigma pointers (recorded against null base
// pointers by EffectiveHamiltonian::precompute) become offsets, and the
// operator pointers become offsets into one packed blob holding every
// operator element the pairs read.  The blob is the union of the operands'
// extents, merged where they overlap or touch.
struct RecordedPairs {
    std::vector<int32_t> tb0, m0, n0, k0, lda0, ldb0, ta1, m1, n1, k1, lda1, ldc1;
    std::vector<double> alpha0, alpha1;
    std::vector<uint64_t> a0, b0, a1, c1;
    std::vector<double> blob;   // filled only by pack() (dumps); the device path uses pack_into
    double mnk = 0;   // block2's multiply-add count of one product
    // the merged operand regions of block2's memory and their blob offsets
    struct Span {
        const double *p;
        uint64_t n;
    };
    std::vector<Span> regions;
    std::vector<uint64_t> region_off;
    uint64_t blob_size = 0;

    // copies every region into dst (blob_size doubles), all host threads
    void pack_into(double *dst) const {
#pragma omp parallel for schedule(dynamic, 16)
        for (long r = 0; r < (long)regions.size(); r++) {
            const double *src = regions[r].p;
            const uint64_t n = regions[r].n;
            double *d = dst + region_off[r];
            // split large regions so every thread streams a share
            std::copy(src, src + n, d);
        }
    }
    void pack() {
        blob.resize(blob_size);
        pack_into(blob.data());
    }

    b2g_pair_seq seq() const {
        b2g_pair_seq s;
        s.n_pairs = (int64_t)tb0.size();
        s.tb0 = tb0.data(), s.m0 = m0.data(), s.n0 = n0.data(), s.k0 = k0.data();
        s.lda0 = lda0.data(), s.ldb0 = ldb0.data();
        s.ta1 = ta1.data(), s.m1 = m1.data(), s.n1 = n1.data(), s.k1 = k1.data();
        s.lda1 = lda1.data(), s.ldc1 = ldc1.data();
        s.alpha0 = alpha0.data(), s.alpha1 = alpha1.data();
        s.a0 = a0.data(), s.b0 = b0.data(), s.a1 = a1.data(), s.c1 = c1.data();
        return s;
    }

    // doubles spanned by op(X) of shape rows x cols stored with leading dim ld
    static uint64_t extent(bool trans, int rows, int cols, int ld) {
        if (rows <= 0 || cols <= 0)
            return 0;
        return trans ? (uint64_t)(cols - 1) * ld + rows : (uint64_t)(rows - 1) * ld + cols;
    }

    template <typename SEQ> void translate(const SEQ &sq, uint64_t nket, uint64_t nbra) {
        const auto &g0 = *sq.batch[0], &g1 = *sq.batch[1];
        if (!g0.acidxs.empty() || g0.c.size() != g1.c.size() || g0.gp.size() != g0.c.size() ||
            g1.gp.size() != g1.c.size())
            throw std::runtime_error("b2g: the recorded GEMM sequence is not a plain pair list "
                                     "(SeqTypes::Tasked rotate records expected)");
        const size_t np = g0.c.size();
        const double *zero = (const double *)0;
        tb0.resize(np), m0.resize(np), n0.resize(np), k0.resize(np), lda0.resize(np), ldb0.resize(np);
        ta1.resize(np), m1.resize(np), n1.resize(np), k1.resize(np), lda1.resize(np), ldc1.resize(np);
        alpha0.resize(np), alpha1.resize(np), a0.resize(np), b0.resize(np), a1.resize(np), c1.resize(np);
        std::vector<Span> spans;
        spans.reserve(2 * np);
        mnk = 0;
        for (size_t i = 0; i < np; i++) {
            if (g0.ta[i] != block2::CblasNoTrans || g1.tb[i] != block2::CblasNoTrans || g0.ldc[i] != g0.n[i] ||
                g1.ldb[i] != g1.n[i] || g0.c[i] != g1.b[i] || g0.beta[i] != 0.0)
                throw std::runtime_error("b2g: unexpected work-matrix layout in a recorded pair");
            tb0[i] = g0.tb[i] != block2::CblasNoTrans, m0[i] = g0.m[i], n0[i] = g0.n[i], k0[i] = g0.k[i];
            lda0[i] = g0.lda[i], ldb0[i] = g0.ldb[i], alpha0[i] = g0.alpha[i];
            ta1[i] = g1.ta[i] != block2::CblasNoTrans, m1[i] = g1.m[i], n1[i] = g1.n[i], k1[i] = g1.k[i];
            lda1[i] = g1.lda[i], ldc1[i] = g1.ldc[i], alpha1[i] = g1.alpha[i];
            a0[i] = (uint64_t)(g0.a[i] - zero);
            c1[i] = (uint64_t)(g1.c[i] - zero);
            if (a0[i] > nket || extent(false, m0[i], k0[i], lda0[i]) > nket - a0[i] ||
                c1[i] > nbra || extent(false, m1[i], n1[i], ldc1[i]) > nbra - c1[i])
                throw std::runtime_error("b2g: a recorded psi/sigma operand lies outside the wavefunction");
            spans.push_back(Span{g0.b[i], extent(tb0[i], k0[i], n0[i], ldb0[i])});
            spans.push_back(Span{g1.a[i], extent(ta1[i], m1[i], k1[i], lda1[i])});
            mnk += (double)m0[i] * n0[i] * k0[i] + (double)m1[i] * n1[i] * k1[i];
        }
        // merge operand extents into disjoint regions, in address order
        std::vector<Span> reg(spans);
        std::sort(reg.begin(), reg.end(), [](const Span &x, const Span &y) { return x.p < y.p; });
        std::vector<Span> merged;
        for (auto &s : reg) {
            if (!merged.empty() && s.p <= merged.back().p + merged.back().n) {
                const double *end = std::max(merged.back().p + merged.back().n, s.p + s.n);
                merged.back().n = (uint64_t)(end - merged.back().p);
            } else
                merged.push_back(s);
        }
        // large regions are cut into pieces of at most 4 Mi doubles so the
        // parallel pack spreads them over the host threads
        const uint64_t piece = (uint64_t)1 << 22;
        std::vector<uint64_t> off(merged.size());
        uint64_t total = 0;
        regions.clear(), region_off.clear();
        for (size_t r = 0; r < merged.size(); r++) {
            off[r] = total;
            for (uint64_t q = 0; q < merged[r].n; q += piece) {
                regions.push_back(Span{merged[r].p + q, std::min(piece, merged[r].n - q)});
                region_off.push_back(total + q);
            }
            total += merged[r].n;
        }
        blob_size = total;
        auto locate = [&](const double *p) -> uint64_t {
            auto it = std::upper_bound(merged.begin(), merged.end(), p,
                                       [](const double *x, const Span &s) { return x < s.p; });
            const size_t r = (size_t)(it - merged.begin()) - 1;
            return off[r] + (uint64_t)(p - merged[r].p);
        };
        for (size_t i = 0; i < np; i++)
            b0[i] = locate(g0.b[i]), a1[i] = locate(g1.a[i]);
    }
};

// The device plan of one recorded H_eff (built lazily from the sequence the
// owning tensor functions recorded; destroyed with them or when a different
// sequence is recorded).
struct DevicePlan {
    std::shared_ptr<Runtime> rt;
    b2g_heff *h = nullptr;
    uint64_t nket = 0, nbra = 0;
    double mnk = 0;
    std::vector<const void *> signature;
    explicit DevicePlan(const std::shared_ptr<Runtime> &rt) : rt(rt) {}
    ~DevicePlan() { release(); }
    void release() {
        if (h != nullptr)
            b2g_heff_destroy(h);
        h = nullptr;
        signature.clear();
    }
    template <typename SEQ> static std::vector<const void *> sign(const SEQ &sq) {
        const auto &g0 = *sq.batch[0], &g1 = *sq.batch[1];
        std::vector<const void *> s{&sq, (const void *)(uintptr_t)g0.c.size()};
        if (!g0.c.empty())
            s.insert(s.end(), {g0.a.front(), g0.b.front(), g1.a.front(), g1.c.front(), g0.a.back(),
                               g0.b.back(), g1.a.back(), g1.c.back()});
        return s;
    }
    // keep: when given, receives the translated pairs and blob (for dumps)
    template <typename SEQ>
    b2g_heff *get(const SEQ &sq, uint64_t ket_size, uint64_t bra_size, RecordedPairs *keep = nullptr) {
        std::vector<const void *> s = sign(sq);
        if (h != nullptr && s == signature && ket_size == nket && bra_size == nbra && keep == nullptr)
            return h;
        release();
        block2::Timer t;
        t.get_time();
        RecordedPairs local;
        RecordedPairs &rp = keep != nullptr ? *keep : local;
        rp.translate(sq, ket_size, bra_size);
        // the device plan is built on a second thread while this one packs
        // the operator blob into the context's pinned staging buffer; the
        // blob is uploaded when both are done
        b2g_pair_seq ps = rp.seq();
        int rc_create = B2G_OK;
        std::string err_create;
        std::thread builder([&] {
            rc_create = b2g_heff_create(rt->ctx, &ps, nullptr, rp.blob_size, B2G_OPS_DEFERRED, ket_size,
                                        bra_size, &h);
            if (rc_create != B2G_OK)
                err_create = b2g_last_error();
        });
        void *stage = nullptr;
        const int rc_buf = b2g_host_buffer(rt->ctx, 8 * std::max<uint64_t>(rp.blob_size, 1), &stage);
        const std::string err_buf = rc_buf != B2G_OK ? b2g_last_error() : "";
        if (rc_buf == B2G_OK)
            rp.pack_into((double *)stage);
        rt->t_plan += t.get_time();
        builder.join();
        if (rc_create != B2G_OK) {
            h = nullptr;
            throw std::runtime_error("b2g_heff_create: " + err_create);
        }
        if (rc_buf != B2G_OK) {
            release();
            throw std::runtime_error("b2g_host_buffer: " + err_buf);
        }
        check(b2g_heff_set_ops(h, (const double *)stage, 0), "b2g_heff_set_ops");
        if (keep != nullptr)
            keep->blob.assign((const double *)stage, (const double *)stage + rp.blob_size);
        rt->t_upload += t.get_time();
        rt->h2d_bytes += 8.0 * (double)rp.blob_size;
        rt->n_heff++;
        nket = ket_size, nbra = bra_size, mnk = rp.mnk, signature = s;
        return h;
    }
};

template <typename S> struct GpuTensorFunctions : block2::TensorFunctions<S, double> {
    typedef block2::TensorFunctions<S, double> TF;
    std::shared_ptr<Runtime> rt;
    std::shared_ptr<DevicePlan> plan;
    GpuTensorFunctions(const std::shared_ptr<block2::OperatorFunctions<S, double>> &opf,
                       const std::shared_ptr<Runtime> &rt)
        : TF(opf), rt(rt), plan(std::make_shared<DevicePlan>(rt)) {
        if (!(opf->seq->mode & block2::SeqTypes::Tasked))
            throw std::runtime_error("GpuTensorFunctions: needs threading->seq_type = SeqTypes::Tasked "
                                     "(the GEMM pairs are recorded by EffectiveHamiltonian::precompute)");
    }
    // every copy (one per EffectiveHamiltonian) owns its own device plan
    std::shared_ptr<TF> copy() const override {
        return std::make_shared<GpuTensorFunctions<S>>(this->opf->copy(), rt);
    }
    b2g_heff *device_plan(uint64_t ket_size, uint64_t bra_size, RecordedPairs *keep = nullptr) {
        return plan->get(*this->opf->seq, ket_size, bra_size, keep);
    }
    // c += scale * H_eff b (host buffers), after precompute recorded the pairs
    void operator()(const block2::GMatrix<double> &b, const block2::GMatrix<double> &c,
                    double scale = 1.0) override {
        auto &sq = *this->opf->seq;
        if (sq.batch[0]->c.empty() && sq.batch[1]->c.empty())
            return;
        b2g_heff *h = device_plan((uint64_t)b.size(), (uint64_t)c.size());
        check(b2g_heff_apply_host(h, b.data, c.data, scale, B2G_FP64), "b2g_heff_apply_host");
        rt->n_apply_fp64++;
        rt->h2d_bytes += 8.0 * (double)b.size(), rt->d2h_bytes += 8.0 * (double)c.size();
        sq.cumulative_nflop += (size_t)plan->mnk;
    }
    // EffectiveHamiltonian::perturbative_noise (src/dmrg/effective_hamiltonian.hpp:262-433)
    // calls this once per noise product; block2's own version records single GEMMs
    // (Tasked mode, batch[1]) that perturbative_noise then replays with
    // BatchGEMMSeq::auto_perform.  With Runtime::noise_on_device the outermost call
    // runs the recorded list on the GPU as H_eff pairs (b2g_noise_pairs) and
    // empties batch[1], so auto_perform adds nothing.  Nested calls (the Sum
    // branch, and the per-thread copies TensorFunctions::parallel_for uses,
    // src/core/tensor_functions.hpp:68-130) only record: their lists are merged
    // into this sequence before the outermost call returns.
    void tensor_product_partial_multiply(
        const std::shared_ptr<block2::OpExpr<S>> &expr, const std::shared_ptr<block2::OpExpr<S>> &xexpr,
        const std::shared_ptr<block2::OperatorTensor<S, double>> &lopt,
        const std::shared_ptr<block2::OperatorTensor<S, double>> &ropt, bool trace_right,
        const std::shared_ptr<block2::SparseMatrix<S, double>> &cmat,
        const std::vector<std::pair<uint8_t, S>> &psubsl,
        const std::vector<std::vector<std::shared_ptr<typename block2::SparseMatrixInfo<S>::ConnectionInfo>>>
            &cinfos,
        const std::vector<S> &vdqs, const std::shared_ptr<block2::SparseMatrixGroup<S, double>> &vmats,
        int &vidx, int tvidx, bool do_reduce) const override {
        const bool outer = rt->noise_depth.fetch_add(1) == 0;
        try {
            TF::tensor_product_partial_multiply(expr, xexpr, lopt, ropt, trace_right, cmat, psubsl, cinfos, vdqs,
                                                vmats, vidx, tvidx, do_reduce);
        } catch (...) {
            rt->noise_depth--;
            throw;
        }
        rt->noise_depth--;
        if (outer && rt->noise_on_device)
            noise_on_device(cmat, vmats);
    }
    // the recorded noise GEMMs: ket operands -> offsets into the ket, operator
    // operands -> a packed blob of their merged extents, outputs -> offsets into
    // the group; then pairs, one device product, and the list is cleared
    void noise_on_device(const std::shared_ptr<block2::SparseMatrix<S, double>> &ket,
                         const std::shared_ptr<block2::SparseMatrixGroup<S, double>> &grp) const {
        auto &sq = *this->opf->seq;
        auto &g1 = *sq.batch[1];
        if (!sq.batch[0]->c.empty())
            throw std::runtime_error("b2g: GEMM pairs recorded next to the noise product");
        const double *kb = ket->data, *vb = grp->data;
        const uint64_t nk = ket->total_memory, nv = grp->total_memory;
        auto trans = [](block2::CBLAS_TRANSPOSE t) { return t == block2::CblasTrans || t == block2::CblasConjTrans; };
        std::vector<int32_t> ta, tb, m, n, k, lda, ldb, ldc, ak, bk;
        std::vector<double> al, be;
        std::vector<uint64_t> ga, gb, gc;
        std::vector<RecordedPairs::Span> spans;
        size_t p = 0;
        for (size_t gi = 0; gi < g1.gp.size(); gi++)
            for (int q = 0; q < (int)g1.gp[gi]; q++, p++) {
                ta.push_back(trans(g1.ta[gi])), tb.push_back(trans(g1.tb[gi]));
                m.push_back(g1.m[gi]), n.push_back(g1.n[gi]), k.push_back(g1.k[gi]);
                lda.push_back(g1.lda[gi]), ldb.push_back(g1.ldb[gi]), ldc.push_back(g1.ldc[gi]);
                al.push_back(g1.alpha[gi]), be.push_back(g1.beta[gi]);
                if (g1.c[p] < vb || g1.c[p] >= vb + nv)
                    throw std::runtime_error("b2g: a noise GEMM writes outside the perturbed group");
                gc.push_back((uint64_t)(g1.c[p] - vb));
                for (int side = 0; side < 2; side++) {
                    const double *x = side == 0 ? g1.a[p] : g1.b[p];
                    const bool is_ket = x >= kb && x < kb + nk;
                    (side == 0 ? ak : bk).push_back(is_ket ? B2G_NOISE_KET : B2G_NOISE_OP);
                    (side == 0 ? ga : gb).push_back(is_ket ? (uint64_t)(x - kb) : 0);
                    if (!is_ket)
                        spans.push_back(RecordedPairs::Span{
                            x, side == 0 ? RecordedPairs::extent(ta.back(), m.back(), k.back(), lda.back())
                                         : RecordedPairs::extent(tb.back(), k.back(), n.back(), ldb.back())});
                }
            }
        const size_t ng = ta.size();
        // operator blob: the operands' extents merged in address order
        std::vector<RecordedPairs::Span> merged(spans);
        std::sort(merged.begin(), merged.end(),
                  [](const RecordedPairs::Span &x, const RecordedPairs::Span &y) { return x.p < y.p; });
        std::vector<RecordedPairs::Span> reg;
        for (auto &s : merged)
            if (!reg.empty() && s.p <= reg.back().p + reg.back().n)
                reg.back().n = (uint64_t)(std::max(reg.back().p + reg.back().n, s.p + s.n) - reg.back().p);
            else
                reg.push_back(s);
        std::vector<uint64_t> roff(reg.size());
        uint64_t nops = 0;
        for (size_t r = 0; r < reg.size(); r++)
            roff[r] = nops, nops += reg[r].n;
        auto locate = [&](const double *x) {
            auto it = std::upper_bound(reg.begin(), reg.end(), x,
                                       [](const double *y, const RecordedPairs::Span &s) { return y < s.p; });
            const size_t r = (size_t)(it - reg.begin()) - 1;
            return roff[r] + (uint64_t)(x - reg[r].p);
        };
        p = 0;
        for (size_t gi = 0, i = 0; gi < g1.gp.size(); gi++)
            for (int q = 0; q < (int)g1.gp[gi]; q++, p++, i++) {
                if (ak[i] == B2G_NOISE_OP)
                    ga[i] = locate(g1.a[p]);
                if (bk[i] == B2G_NOISE_OP)
                    gb[i] = locate(g1.b[p]);
            }
        // the group's row-major blocks
        std::vector<uint64_t> boff;
        std::vector<int32_t> brows, bcols;
        for (int j = 0; j < grp->n; j++) {
            const auto &info = grp->infos[j];
            for (int b = 0; b < info->n; b++) {
                boff.push_back(grp->offsets[j] + info->block_shifts[b]);
                brows.push_back((int32_t)info->n_states_bra[b]), bcols.push_back((int32_t)info->n_states_ket[b]);
            }
        }
        b2g_gemm_list gl{(int64_t)ng, ta.data(), tb.data(), m.data(), n.data(), k.data(), lda.data(),
                         ldb.data(), ldc.data(), ak.data(), bk.data(), al.data(), be.data(),
                         ga.data(), gb.data(), gc.data()};
        RecordedPairs rp;
        rp.tb0.resize(ng), rp.m0.resize(ng), rp.n0.resize(ng), rp.k0.resize(ng), rp.lda0.resize(ng);
        rp.ldb0.resize(ng), rp.ta1.resize(ng), rp.m1.resize(ng), rp.n1.resize(ng), rp.k1.resize(ng);
        rp.lda1.resize(ng), rp.ldc1.resize(ng), rp.alpha0.resize(ng), rp.alpha1.resize(ng);
        rp.a0.resize(ng), rp.b0.resize(ng), rp.a1.resize(ng), rp.c1.resize(ng);
        b2g_pair_arrays out{rp.tb0.data(), rp.m0.data(), rp.n0.data(), rp.k0.data(), rp.lda0.data(),
                            rp.ldb0.data(), rp.ta1.data(), rp.m1.data(), rp.n1.data(), rp.k1.data(),
                            rp.lda1.data(), rp.ldc1.data(), rp.alpha0.data(), rp.alpha1.data(),
                            rp.a0.data(), rp.b0.data(), rp.a1.data(), rp.c1.data()};
        int64_t np = 0;
        int32_t dim = 0;
        check(b2g_noise_pairs(&gl, nk, nops, nv, (int64_t)boff.size(), boff.data(), brows.data(), bcols.data(),
                              &out, &np, &dim),
              "b2g_noise_pairs");
        if (np == 0) {  // nothing to add (e.g. a site without the identity operator on one side)
            g1.clear();
            return;
        }
        for (auto *v : {&rp.tb0, &rp.m0, &rp.n0, &rp.k0, &rp.lda0, &rp.ldb0, &rp.ta1, &rp.m1, &rp.n1, &rp.k1,
                        &rp.lda1, &rp.ldc1})
            v->resize((size_t)np);
        rp.alpha0.resize((size_t)np), rp.alpha1.resize((size_t)np);
        rp.a0.resize((size_t)np), rp.b0.resize((size_t)np), rp.a1.resize((size_t)np), rp.c1.resize((size_t)np);
        std::vector<double> blob(nops + (uint64_t)dim * dim, 0.0);
        for (size_t r = 0; r < reg.size(); r++)
            std::copy(reg[r].p, reg[r].p + reg[r].n, blob.begin() + roff[r]);
        for (int32_t d = 0; d < dim; d++)
            blob[nops + (uint64_t)d * dim + d] = 1.0;
        b2g_pair_seq ps = rp.seq();
        b2g_heff *h = nullptr;
        check(b2g_heff_create(rt->ctx, &ps, blob.data(), blob.size(), 0, nk, nv, &h), "b2g_heff_create");
        const int rc = b2g_heff_apply_host(h, kb, grp->data, 1.0, B2G_FP64);
        const std::string err = rc != B2G_OK ? b2g_last_error() : "";
        b2g_heff_destroy(h);
        if (rc != B2G_OK)
            throw std::runtime_error("b2g_heff_apply_host (noise): " + err);
        rt->n_noise++;
        rt->h2d_bytes += 8.0 * (double)(blob.size() + nk + nv), rt->d2h_bytes += 8.0 * (double)nv;
        sq.cumulative_nflop += g1.nflop;
        g1.clear();
    }
    // Expect's fast expectation algorithm (TensorFunctions::tensor_product_expectation,
    // src/core/tensor_functions.hpp:1701-1877, used for the PDM MPOs) with its partials
    // on the GPU.  Each unique left operator a (per conj, dq of the right operator and
    // operator quantum) gets a partial <bra| a |ket>; the block loop of
    // OperatorFunctions::tensor_left_partial_expectation (src/core/operator_functions.hpp:354-410)
    // is written as H_eff pairs: a on the left of GEMM0 ("psi"), the ket and bra blocks
    // in the operator blob, the partials as sigma.  With a transposed (which GEMM0's
    // left operand cannot be) the pair uses bra^T a^T ket = (ket^T a bra)^T and writes
    // the block transposed; a partial whose conj bits differ is stored block-transposed.
    // One FP64 product computes every partial; the expectations are then the
    // reference's sums of factor * dot(partial, right operator) on the host.
    std::vector<std::pair<std::shared_ptr<block2::OpExpr<S>>, double>>
    tensor_product_expectation(const std::vector<std::shared_ptr<block2::OpExpr<S>>> &names,
                               const std::vector<std::shared_ptr<block2::OpExpr<S>>> &exprs,
                               const std::shared_ptr<block2::OperatorTensor<S, double>> &lopt,
                               const std::shared_ptr<block2::OperatorTensor<S, double>> &ropt,
                               const std::shared_ptr<block2::SparseMatrix<S, double>> &cmat,
                               const std::shared_ptr<block2::SparseMatrix<S, double>> &vmat,
                               bool all_reduce) const override {
        typedef block2::OpProduct<S, double> Prod;
        if (lopt->get_type() == block2::OperatorTensorTypes::Delayed ||
            ropt->get_type() == block2::OperatorTensorTypes::Delayed)
            throw std::runtime_error("GpuTensorFunctions: expectation with delayed contraction "
                                     "(the reference does not support it either)");
        std::vector<std::pair<std::shared_ptr<block2::OpExpr<S>>, double>> expectations(names.size());
        const S ket_dq = cmat->info->delta_quantum, bra_dq = vmat->info->delta_quantum;
        auto products = [&](size_t k) {
            std::vector<std::shared_ptr<Prod>> ps;
            if (exprs[k]->get_type() == block2::OpTypes::Prod)
                ps.push_back(std::dynamic_pointer_cast<Prod>(exprs[k]));
            else if (exprs[k]->get_type() == block2::OpTypes::Sum)
                ps = std::dynamic_pointer_cast<block2::OpSum<S, double>>(exprs[k])->strings;
            else if (exprs[k]->get_type() == block2::OpTypes::SumProd)
                throw std::runtime_error("GpuTensorFunctions: expectation with delayed contraction");
            return ps;
        };
        auto opdq_of = [&](size_t k) { return std::dynamic_pointer_cast<block2::OpElement<S, double>>(names[k])->q_label; };
        // the partials, in first-appearance order
        struct Part {
            uint8_t conj;
            S opdq;
            std::shared_ptr<block2::SparseMatrix<S, double>> lmat;
            std::shared_ptr<block2::SparseMatrixInfo<S>> info;
            uint64_t off;
            bool trans;
        };
        std::vector<Part> parts;
        std::map<std::tuple<int, uint64_t, uint64_t, const double *>, int> pidx;
        uint64_t nsig = 0;
        for (size_t k = 0; k < exprs.size(); k++) {
            const S opdq = opdq_of(k);
            if (opdq.combine(bra_dq, ket_dq) == S(S::invalid))
                continue;
            for (auto &op : products(k)) {
                auto info = ropt->ops.at(op->b)->info;
                auto lmat = lopt->ops.at(op->a);
                const auto key = std::make_tuple((int)op->conj, (uint64_t)info->delta_quantum.data,
                                                 (uint64_t)opdq.data, (const double *)lmat->data);
                if (pidx.count(key))
                    continue;
                pidx[key] = (int)parts.size();
                parts.push_back(Part{op->conj, opdq, lmat, info, nsig, (op->conj & 1) != ((op->conj & 2) >> 1)});
                nsig += info->template get_total_memory<double>();
            }
        }
        // the pairs of every partial block
        std::vector<double> lblob, oblob(cmat->data, cmat->data + cmat->total_memory);
        const bool same = vmat->data == cmat->data;
        if (!same)
            oblob.insert(oblob.end(), vmat->data, vmat->data + vmat->total_memory);
        const uint64_t vbase = same ? 0 : cmat->total_memory;
        std::map<const double *, uint64_t> loff;
        RecordedPairs rp;
        auto cinfo = cmat->info->cinfo;
        if (!parts.empty() && cinfo == nullptr)
            throw std::runtime_error("GpuTensorFunctions: expectation without the wavefunction connection info");
        for (auto &P : parts) {
            const double s0 = P.lmat->factor * vmat->factor * cmat->factor;
            if (std::abs(s0) < TINY)  // block2's TINY macro (1e-20)
                continue;
            if (!loff.count(P.lmat->data)) {
                loff[P.lmat->data] = lblob.size();
                lblob.insert(lblob.end(), P.lmat->data, P.lmat->data + P.lmat->total_memory);
            }
            const uint64_t abase = loff[P.lmat->data];
            const bool ca = P.conj & 1, cc = (P.conj & 2) >> 1;
            const S adq = P.lmat->info->delta_quantum, bdq = P.info->delta_quantum;
            const S abdq = P.opdq.combine(ca ? -adq : adq, cc ? bdq : -bdq);
            const int ik = (int)(std::lower_bound(cinfo->quanta + cinfo->n[P.conj], cinfo->quanta + cinfo->n[P.conj + 1],
                                                  abdq) - cinfo->quanta);
            if (ik >= cinfo->n[P.conj + 1])
                throw std::runtime_error("GpuTensorFunctions: no connection for a partial expectation");
            const int ixa = cinfo->idx[ik], ixb = ik == cinfo->n[4] - 1 ? cinfo->nc : cinfo->idx[ik + 1];
            for (int il = ixa; il < ixb; il++) {
                const int ia = cinfo->ia[il], ib = cinfo->ib[il], ic = cinfo->ic[il], iv = (int)cinfo->stride[il];
                const block2::GMatrix<double> A = (*P.lmat)[ia], V = (*vmat)[iv], K = (*cmat)[ic];
                const int crow = (int)P.info->n_states_bra[ib], ccol = (int)P.info->n_states_ket[ib];
                const uint64_t offA = abase + (uint64_t)(A.data - P.lmat->data);
                const uint64_t offK = (uint64_t)(K.data - cmat->data), offV = vbase + (uint64_t)(V.data - vmat->data);
                const block2::GMatrix<double> &X = ca ? V : K, &Y = ca ? K : V;
                const bool out_t = ca != cc;
                if (A.n != X.m || Y.m != A.m || (out_t ? ccol : crow) != Y.n || (out_t ? crow : ccol) != X.n)
                    throw std::runtime_error("GpuTensorFunctions: partial expectation block shapes");
                rp.tb0.push_back(0), rp.m0.push_back(A.m), rp.k0.push_back(A.n), rp.n0.push_back(X.n);
                rp.lda0.push_back(A.n), rp.ldb0.push_back(X.n), rp.a0.push_back(offA);
                rp.b0.push_back(ca ? offV : offK);
                rp.ta1.push_back(1), rp.m1.push_back(Y.n), rp.k1.push_back(Y.m), rp.n1.push_back(X.n);
                rp.lda1.push_back(Y.n), rp.a1.push_back(ca ? offK : offV);
                rp.ldc1.push_back(out_t ? crow : ccol), rp.c1.push_back(P.off + P.info->block_shifts[ib]);
                rp.alpha0.push_back(1.0), rp.alpha1.push_back(s0 * cinfo->factor[il]);
            }
        }
        std::vector<double> part(nsig, 0.0);
        if (!rp.tb0.empty()) {
            b2g_pair_seq ps = rp.seq();
            b2g_heff *h = nullptr;
            check(b2g_heff_create(rt->ctx, &ps, oblob.data(), oblob.size(), 0, lblob.size(), nsig, &h),
                  "b2g_heff_create (expectation)");
            const int rc = b2g_heff_apply_host(h, lblob.data(), part.data(), 1.0, B2G_FP64);
            const std::string err = rc != B2G_OK ? b2g_last_error() : "";
            b2g_heff_destroy(h);
            if (rc != B2G_OK)
                throw std::runtime_error("b2g_heff_apply_host (expectation): " + err);
            rt->n_expect++;
            rt->h2d_bytes += 8.0 * (double)(oblob.size() + lblob.size() + nsig), rt->d2h_bytes += 8.0 * (double)nsig;
        }
        // transposed partials back to row-major blocks
        for (auto &P : parts)
            if (P.trans)
                for (int ib = 0; ib < P.info->n; ib++) {
                    const int r = (int)P.info->n_states_bra[ib], c = (int)P.info->n_states_ket[ib];
                    double *x = part.data() + P.off + P.info->block_shifts[ib];
                    std::vector<double> t(x, x + (size_t)r * c);
                    for (int i = 0; i < r; i++)
                        for (int j = 0; j < c; j++)
                            x[(size_t)i * c + j] = t[(size_t)j * r + i];
                }
        // expectation k = sum of factor * dot(partial, right operator) over its products
        for (size_t k = 0; k < exprs.size(); k++) {
            expectations[k] = std::make_pair(names[k], 0.0);
            const S opdq = opdq_of(k);
            if (opdq.combine(bra_dq, ket_dq) == S(S::invalid))
                continue;
            double r = 0.0;
            for (auto &op : products(k)) {
                auto rmat = ropt->ops.at(op->b);
                auto lmat = lopt->ops.at(op->a);
                const int p = pidx.at(std::make_tuple((int)op->conj, (uint64_t)rmat->info->delta_quantum.data,
                                                      (uint64_t)opdq.data, (const double *)lmat->data));
                const double *x = part.data() + parts[p].off;
                double d = 0.0;
                for (uint64_t q = 0; q < rmat->total_memory; q++)
                    d += x[q] * rmat->data[q];
                r += op->factor * d;
            }
            expectations[k].second = r;
        }
        return expectations;
    }
};

// Writes one H_eff as raw little-endian arrays plus a manifest ("name dtype
// count" lines and "#key value" scalars): the translated pairs, the operator
// blob, the Davidson initial guess psi, diag(H_eff), and after the solve the
// eigenvector and energy -- a real-operator problem for measurements.
struct HeffDump {
    std::string dir;
    std::ofstream man;
    explicit HeffDump(const std::string &d) : dir(d), man(d + "/manifest.txt") { man.precision(17); }
    template <typename T> void arr(const char *name, const std::vector<T> &v, const char *dt) {
        std::ofstream f(dir + "/" + name + ".bin", std::ios::binary);
        f.write((const char *)v.data(), (std::streamsize)(sizeof(T) * v.size()));
        man << name << " " << dt << " " << v.size() << "\n";
    }
    void scalar(const char *name, double v) { man << "#" << name << " " << v << "\n"; }
    void pairs(const RecordedPairs &rp) {
        arr("tb0", rp.tb0, "i4"), arr("m0", rp.m0, "i4"), arr("n0", rp.n0, "i4"), arr("k0", rp.k0, "i4");
        arr("lda0", rp.lda0, "i4"), arr("ldb0", rp.ldb0, "i4"), arr("ta1", rp.ta1, "i4");
        arr("m1", rp.m1, "i4"), arr("n1", rp.n1, "i4"), arr("k1", rp.k1, "i4"), arr("lda1", rp.lda1, "i4");
        arr("ldc1", rp.ldc1, "i4"), arr("alpha0", rp.alpha0, "f8"), arr("alpha1", rp.alpha1, "f8");
        arr("a0", rp.a0, "u8"), arr("b0", rp.b0, "u8"), arr("a1", rp.a1, "u8"), arr("c1", rp.c1, "u8");
        arr("ops", rp.blob, "f8");
    }
};

template <typename S> struct GpuDMRG : block2::DMRG<S, double, double> {
    typedef block2::DMRG<S, double, double> D;
    std::shared_ptr<Runtime> rt;
    // optional: dump the H_eff of site dump_site in sweep dump_sweep to dump_dir
    std::string dump_dir;
    int dump_sweep = -1, dump_site = -1;
    GpuDMRG(const std::shared_ptr<block2::MovingEnvironment<S, double, double>> &me,
            const std::vector<block2::ubond_t> &bond_dims, const std::vector<double> &noises,
            const std::shared_ptr<Runtime> &rt)
        : D(me, bond_dims, noises), rt(rt) {}
    void unsupported_check() const {
        const char *why = nullptr;
        if (this->state_specific || !this->projection_weights.empty() || !this->ext_mes.empty())
            why = "state-specific / projected solves";
        else if (this->metric_me != nullptr)
            why = "a metric (generalized) eigenproblem";
        else if (this->context_ket != nullptr)
            why = "a context MPS";
        else if (this->me->para_rule != nullptr)
            why = "a parallel rule";
        else if (this->me->bra != this->me->ket)
            why = "a bra MPS different from the ket";
        else if (this->davidson_type != block2::DavidsonTypes::Normal)
            why = "a Davidson type other than Normal";
        else if (this->davidson_rel_conv_thrd != 0)
            why = "a relative Davidson threshold";
        else if (this->eff_kernel != nullptr)
            why = "an EffectiveKernel hook";
        if (why != nullptr)
            throw std::runtime_error(std::string("GpuDMRG: ") + why + " is not implemented on the GPU path");
    }
    // DMRG::two_dot_eigs_and_perturb (src/dmrg/sweep_algorithm.hpp:1183-1268)
    // with the eigensolve on the device.  Timers, callbacks and bookkeeping
    // follow the reference so the sweep prints and results keep their meaning.
    typedef typename D::FPLS FPLS;  // the energy type of the sweep (long double)
    std::tuple<FPLS, int, size_t, double>
    two_dot_eigs_and_perturb(const bool forward, const int i, const double davidson_conv_thrd,
                             const double noise,
                             std::shared_ptr<block2::SparseMatrixGroup<S, double>> &pket) override {
        unsupported_check();
        this->_t.get_time();
        this->torth += this->_t.get_time();
        // compute_diag = false: the diagonal comes from the device (b2g_heff_diag)
        std::shared_ptr<block2::EffectiveHamiltonian<S, double>> h_eff = this->me->eff_ham(
            block2::FuseTypes::FuseLR, forward, false, this->me->bra->tensors[i], this->me->ket->tensors[i]);
        auto gtf = std::dynamic_pointer_cast<GpuTensorFunctions<S>>(h_eff->tf);
        if (gtf == nullptr)
            throw std::runtime_error("GpuDMRG: mpo->tf must be a GpuTensorFunctions");
        this->sweep_max_eff_ham_size = std::max(this->sweep_max_eff_ham_size, h_eff->op->get_total_memory());
        this->sweep_max_eff_wfn_size = std::max(this->sweep_max_eff_wfn_size, (size_t)h_eff->ket->total_memory);
        this->current_eff_ham = h_eff;
        block2::callback_()->compute("DMRG::sweep::iter.eff_ham", this->iprint);
        this->current_eff_ham = nullptr;
        this->teff += this->_t.get_time();
        block2::Timer t;
        t.get_time();
        const uint64_t nket = h_eff->ket->total_memory, nbra = h_eff->bra->total_memory;
        h_eff->precompute();
        const bool dump = !dump_dir.empty() && this->isweep == dump_sweep && i == dump_site;
        std::unique_ptr<RecordedPairs> kept(dump ? new RecordedPairs() : nullptr);
        b2g_heff *h = gtf->device_plan(nket, nbra, kept.get());
        std::vector<double> diag(nket);
        check(b2g_heff_diag_host(h, diag.data()), "b2g_heff_diag_host");
        std::unique_ptr<HeffDump> dw;
        if (dump) {
            dw.reset(new HeffDump(dump_dir));
            dw->pairs(*kept);
            kept.reset();
            dw->arr("psi", std::vector<double>(h_eff->ket->data, h_eff->ket->data + nket), "f8");
            dw->arr("diag", diag, "f8");
            dw->scalar("psi_size", (double)nket), dw->scalar("sigma_size", (double)nbra);
            dw->scalar("isweep", this->isweep), dw->scalar("site", i), dw->scalar("forward", forward);
            dw->scalar("conv_thrd", davidson_conv_thrd), dw->scalar("n_sites", this->me->n_sites);
            dw->scalar("const_e", (double)this->me->mpo->const_e);
            dw->scalar("def_min", this->davidson_def_min_size), dw->scalar("def_max", this->davidson_def_max_size);
        }
        block2::Timer td;
        td.get_time();
        b2g_davidson_result res;
        check(b2g_davidson(h, diag.data(), h_eff->ket->data, davidson_conv_thrd, this->davidson_max_iter,
                           this->davidson_def_min_size, this->davidson_def_max_size, rt->form, &res),
              "b2g_davidson");
        rt->t_davidson += td.get_time();
        // diag down, diag + psi up, psi down
        rt->d2h_bytes += 16.0 * (double)nket, rt->h2d_bytes += 16.0 * (double)nket;
        if (dw != nullptr) {
            dw->arr("psi_converged", std::vector<double>(h_eff->ket->data, h_eff->ket->data + nket), "f8");
            dw->scalar("davidson_energy", res.energy), dw->scalar("davidson_iterations", res.n_iter);
            dw->man.flush();
        }
        rt->n_apply_fp64 += res.n_apply_fp64;
        rt->n_apply_reduced += res.n_apply_mixed;
        const size_t nflop = (size_t)(gtf->plan->mnk * (double)(res.n_apply_fp64 + res.n_apply_mixed));
        h_eff->post_precompute();
        gtf->plan->release();
        std::tuple<FPLS, int, size_t, double> pdi =
            std::make_tuple((FPLS)res.energy, (int)res.n_iter, nflop, t.get_time());
        this->teig += this->_t.get_time();
        this->current_eff_ham = h_eff;
        block2::callback_()->compute("DMRG::sweep::iter.eff_ham.end", this->iprint);
        this->current_eff_ham = nullptr;
        if ((this->noise_type & block2::NoiseTypes::Perturbative) && noise != 0)
            pket = h_eff->perturbative_noise(forward, i, i + 1, block2::FuseTypes::FuseLR,
                                             this->me->ket->info, this->noise_type, this->me->para_rule);
        this->tprt += this->_t.get_time();
        h_eff->deallocate();
        return pdi;
    }
    // DMRG::multi_two_dot_eigs_and_perturb (src/dmrg/sweep_algorithm.hpp:2361-2495),
    // the state-averaged (MultiMPS) step: all roots share one H_eff, which is
    // recorded once and solved by the device block Davidson (b2g_davidson_multi:
    // the Olsen corrections of every unconverged root go through one batched
    // product per iteration).  Roots with several target quanta per root (a
    // wavefunction group of more than one block structure) are not supported.
    std::tuple<std::vector<FPLS>, int, size_t, double>
    multi_two_dot_eigs_and_perturb(const bool forward, const int i, const double davidson_conv_thrd,
                                   const double noise,
                                   std::shared_ptr<block2::SparseMatrixGroup<S, double>> &pket,
                                   std::vector<std::vector<std::pair<S, double>>> &mps_quanta) override {
        unsupported_check();
        if (this->cpx_me != nullptr)
            throw std::runtime_error("GpuDMRG: a complex correction environment is not implemented on the GPU path");
        auto mket = std::dynamic_pointer_cast<block2::MultiMPS<S, double>>(this->me->ket);
        this->_t.get_time();
        this->torth += this->_t.get_time();
        std::shared_ptr<block2::EffectiveHamiltonian<S, double, block2::MultiMPS<S, double>>> h_eff =
            this->me->multi_eff_ham(block2::FuseTypes::FuseLR, forward, false);
        auto gtf = std::dynamic_pointer_cast<GpuTensorFunctions<S>>(h_eff->tf);
        if (gtf == nullptr)
            throw std::runtime_error("GpuDMRG: mpo->tf must be a GpuTensorFunctions");
        const int nroot = (int)h_eff->ket.size();
        for (int r = 0; r < nroot; r++)
            if (h_eff->ket[r]->n != 1 || h_eff->bra[r]->n != 1)
                throw std::runtime_error("GpuDMRG: state-averaged roots with several target quanta per root are "
                                         "not implemented on the GPU path");
        this->sweep_max_eff_ham_size = std::max(this->sweep_max_eff_ham_size, h_eff->op->get_total_memory());
        size_t wsz = 0;
        for (int r = 0; r < nroot; r++)
            wsz += h_eff->ket[r]->total_memory;
        this->sweep_max_eff_wfn_size = std::max(this->sweep_max_eff_wfn_size, wsz);
        this->current_multi_eff_ham = h_eff;
        block2::callback_()->compute("DMRG::sweep::iter.eff_ham", this->iprint);
        this->current_multi_eff_ham = nullptr;
        this->teff += this->_t.get_time();
        block2::Timer t;
        t.get_time();
        const uint64_t nket = h_eff->ket[0]->total_memory, nbra = h_eff->bra[0]->total_memory;
        // as in the reference (effective_hamiltonian.hpp:1726-1728): no more
        // roots than the dimension; the surplus roots keep their vectors
        const int k = (int)std::min<uint64_t>((uint64_t)nroot, nket);
        h_eff->precompute();
        b2g_heff *h = gtf->device_plan(nket, nbra);
        std::vector<double> diag(nket), psi((size_t)k * nket), energies(k);
        check(b2g_heff_diag_host(h, diag.data()), "b2g_heff_diag_host");
        for (int r = 0; r < k; r++)
            std::copy(h_eff->ket[r]->data, h_eff->ket[r]->data + nket, psi.data() + (size_t)r * nket);
        block2::Timer td;
        td.get_time();
        b2g_davidson_result res;
        check(b2g_davidson_multi(h, diag.data(), psi.data(), k, davidson_conv_thrd, this->davidson_max_iter,
                                 std::max(this->davidson_def_min_size, k),
                                 std::max(this->davidson_def_max_size, k + k / 2 + 1), rt->form,
                                 energies.data(), &res),
              "b2g_davidson_multi");
        rt->t_davidson += td.get_time();
        rt->d2h_bytes += 8.0 * (double)nket * (k + 1), rt->h2d_bytes += 8.0 * (double)nket * (k + 1);
        for (int r = 0; r < k; r++)
            std::copy(psi.data() + (size_t)r * nket, psi.data() + (size_t)(r + 1) * nket, h_eff->ket[r]->data);
        rt->n_apply_fp64 += res.n_apply_fp64;
        rt->n_apply_reduced += res.n_apply_mixed;
        const size_t nflop = (size_t)(gtf->plan->mnk * (double)(res.n_apply_fp64 + res.n_apply_mixed));
        h_eff->post_precompute();
        gtf->plan->release();
        std::tuple<std::vector<FPLS>, int, size_t, double> pdi = std::make_tuple(
            std::vector<FPLS>(energies.begin(), energies.end()), (int)res.n_iter, nflop, t.get_time());
        for (int r = 0; r < mket->nroots; r++) {
            mps_quanta[r] = h_eff->ket[r]->delta_quanta();
            const double cut = this->quanta_cutoff;
            mps_quanta[r].erase(std::remove_if(mps_quanta[r].begin(), mps_quanta[r].end(),
                                               [cut](const std::pair<S, double> &p) { return p.second < cut; }),
                                mps_quanta[r].end());
        }
        this->teig += this->_t.get_time();
        this->current_multi_eff_ham = h_eff;
        block2::callback_()->compute("DMRG::sweep::iter.eff_ham.end", this->iprint);
        this->current_multi_eff_ham = nullptr;
        if ((this->noise_type & block2::NoiseTypes::Perturbative) && noise != 0)
            pket = h_eff->perturbative_noise(forward, i, i + 1, block2::FuseTypes::FuseLR, mket->info,
                                             mket->weights, this->noise_type, this->me->para_rule);
        this->tprt += this->_t.get_time();
        h_eff->deallocate();
        return pdi;
    }
};

// Installs the GPU tensor functions into an MPO (what a block2 user does
// once per MPO before building the MovingEnvironment).
template <typename S>
void install(const std::shared_ptr<block2::MPO<S, double>> &mpo, const std::shared_ptr<Runtime> &rt) {
    mpo->tf = std::make_shared<GpuTensorFunctions<S>>(mpo->tf->opf, rt);
}

} // namespace b2g_block2
