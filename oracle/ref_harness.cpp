// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY (never shipped, never measured).
//
// Drives the reference's own CPU implementation of two-site DMRG (block2,
// header-only build against the reference's src/ directory, not vendored) and
// writes, for selected sites of selected sweeps, everything the GPU hot path
// must reproduce:
//
//   * the recorded GEMM-pair sequence of H_eff*psi, exactly as
//     EffectiveHamiltonian::precompute (src/dmrg/effective_hamiltonian.hpp:226-246)
//     leaves it in BatchGEMMSeq::batch[0] / batch[1]
//     (src/core/batch_gemm.hpp:847-1707), with every operator pointer
//     translated into an offset of a packed operator blob;
//   * the packed operator blob itself (all L/R block data those pairs read);
//   * psi (the two-site wavefunction entering Davidson), sigma = H_eff*psi
//     computed by the reference's Tasked replay (batch_gemm.hpp:1613-1689),
//     diag(H_eff) (effective_hamiltonian.hpp:172-182);
//   * after Davidson: the converged psi and its energy;
//   * optionally the perturbative-noise product of that converged psi
//     (EffectiveHamiltonian::perturbative_noise, --noise-product): the single
//     GEMMs it records, the operator blob they read and the reference's
//     perturbed-wavefunction group;
//   * per sweep: energies, discarded weights, bond dimensions.
//
// Output: one directory per dumped site, holding raw little-endian arrays and
// a manifest.txt ("name dtype count" lines, "#key value" scalars).
// Build recipe: oracle/build_ref.sh. Fixture conversion: tests/golden/make_fixtures.py.

#include "block2_core.hpp"
#include "block2_dmrg.hpp"
#include <sys/stat.h>
#include <functional>
#include <mutex>

using namespace block2;

namespace harness {

struct Opts {
    string ham = "hubbard";   // "hubbard" or a FCIDUMP path
    int L = 8;                // hubbard sites
    double t = 1.0, U = 4.0;  // hubbard parameters
    string sym = "su2";       // su2 | sz
    int M = 100, nsweeps = 4, nthreads = 4, seed = 0;
    vector<double> noises = {0.0};
    vector<double> dav_thrds = {1e-10};
    double tol = 0.0;
    string out = "b2g_dump";  // --out: dump directory (relative to the working directory)
    int dump_sweep = 0;       // -1: all sweeps
    int dump_site = -1;       // -1: middle site (n/2-1); -2: all sites
    bool with_data = true;    // false: structure only (no operator blob)
    bool dump_dm = true;      // density-matrix / split data after Davidson
    bool effprob = false;     // also the reference's EffectiveProblem export of the dumped H_eff
    int noise = 0;            // also the perturbative-noise product of the dumped site's converged ket:
                              // 1 = NoiseTypes::ReducedPerturbative, else that NoiseTypes value
    // after the run: the reference's 1-/2-PDM of the final MPS, and for each
    // listed FCIDUMP the H_eff at the final MPS's centre with that Hamiltonian
    // (first site of one sweep on a copy of the final MPS: fixed MPS)
    bool pdm = false;
    vector<string> perturb;
    int perturb_site = -1;    // centre moved here first (-1: n/2 - 1)
    int perturb_threads = 0;  // threads of the perturbed walks (0: --threads); 1 gives every
                              // perturbed H_eff the same GEMM pair order
    int npdm_call = -1;       // with --pdm: record the C-th fast expectation of the PDM sweep
    int npdm_order = 1;       // of the 1-PDM (1) or the 2-PDM (2) sweep
};

static void mkdirs(const string &p) {
    string cur;
    for (size_t i = 0; i < p.size(); i++) {
        cur.push_back(p[i]);
        if (p[i] == '/' || i + 1 == p.size())
            mkdir(cur.c_str(), 0755);
    }
}

struct Writer {
    string dir;
    ofstream man;
    explicit Writer(const string &d) : dir(d) {
        mkdirs(d);
        man.open(d + "/manifest.txt");
        man << setprecision(17);
    }
    template <typename T>
    void arr(const string &name, const T *p, size_t n, const char *dtype) {
        ofstream f(dir + "/" + name + ".bin", ios::binary);
        f.write((const char *)p, sizeof(T) * n);
        man << name << " " << dtype << " " << n << "\n";
    }
    template <typename T>
    void vec(const string &name, const vector<T> &v, const char *dtype) {
        arr(name, v.data(), v.size(), dtype);
    }
    void scalar(const string &name, double v) { man << "#" << name << " " << v << "\n"; }
};

// one contiguous operator data region (SparseMatrix::data, total_memory)
struct Region {
    const double *p;
    size_t n;
    size_t blob_off = 0;
    bool used = false;
};

// Perturbative-noise recorder.  In Tasked mode
// EffectiveHamiltonian::perturbative_noise (src/dmrg/effective_hamiltonian.hpp:262-433)
// records single GEMMs c += alpha op(a) op(b) into BatchGEMMSeq::batch[1]
// (BatchGEMMSeq::multiply, three_rotate_tr_left/right, src/core/batch_gemm.hpp:887-891,
// 1025-1107, and AdvancedGEMM::multiply's per-row form, batch_gemm.hpp:584-607),
// one operand a ket block, the other an operator block, c a block of the
// perturbed-wavefunction group.  Each OperatorFunctions call that adds GEMMs is
// followed here by reading the new entries; operand matrices that the
// H_eff's operator tensors do not hold (built on the fly from a delayed
// expression and freed after recording) are copied while they are alive.
struct NoiseRecorder {
    struct Gemm {
        bool ta, tb;
        int m, n, k, lda, ldb, ldc;
        double alpha, beta;
        const double *a, *b;
        double *c;
        int a_held = -1, b_held = -1;  // index into held (else: H_eff operator or ket)
        size_t a_off = 0, b_off = 0;   // offset within the held copy
    };
    std::mutex mu;
    const double *ket = nullptr;
    size_t nket = 0;
    std::function<bool(const double *, size_t)> known;  // inside an H_eff operator
    // batch[1] groups / entries already read.  With more than one thread,
    // TensorFunctions::parallel_for records into per-thread copies of the
    // sequence and merges them (src/core/tensor_functions.hpp:68-130), so the
    // recorder requires one sequence: run it with --threads 1.
    const BatchGEMM<double> *src = nullptr;
    size_t g_done = 0, p_done = 0;
    vector<Gemm> gemms;
    vector<vector<double>> held;
    static bool trans(CBLAS_TRANSPOSE t) { return t == CblasTrans || t == CblasConjTrans; }
    static size_t extent(bool t, int rows, int cols, int ld) {
        if (rows == 0 || cols == 0)
            return 0;
        return t ? (size_t)(cols - 1) * ld + rows : (size_t)(rows - 1) * ld + cols;
    }
    void take(const BatchGEMM<double> &bt, const vector<pair<const double *, size_t>> &mats) {
        lock_guard<std::mutex> lk(mu);
        map<const double *, int> copied;  // operand matrix -> held index (this call)
        auto place = [&](const double *p, size_t ext, int &hi, size_t &off) {
            if ((p >= ket && p + ext <= ket + nket) || known(p, ext))
                return;
            for (auto &mm : mats)
                if (p >= mm.first && p + ext <= mm.first + mm.second) {
                    auto it = copied.find(mm.first);
                    if (it == copied.end()) {
                        held.emplace_back(mm.first, mm.first + mm.second);
                        it = copied.emplace(mm.first, (int)held.size() - 1).first;
                    }
                    hi = it->second, off = (size_t)(p - mm.first);
                    return;
                }
            throw runtime_error("noise recorder: operand outside the ket, the operators and the call's matrices");
        };
        if (src != nullptr && src != &bt)
            throw runtime_error("noise recorder: GEMMs recorded into two sequences (use --threads 1)");
        src = &bt;
        for (; g_done < bt.gp.size(); g_done++)
            for (MKL_INT q = 0; q < bt.gp[g_done]; q++, p_done++) {
                Gemm g;
                g.ta = trans(bt.ta[g_done]), g.tb = trans(bt.tb[g_done]);
                g.m = bt.m[g_done], g.n = bt.n[g_done], g.k = bt.k[g_done];
                g.lda = bt.lda[g_done], g.ldb = bt.ldb[g_done], g.ldc = bt.ldc[g_done];
                g.alpha = bt.alpha[g_done], g.beta = bt.beta[g_done];
                g.a = bt.a[p_done], g.b = bt.b[p_done], g.c = bt.c[p_done];
                place(g.a, extent(g.ta, g.m, g.k, g.lda), g.a_held, g.a_off);
                place(g.b, extent(g.tb, g.k, g.n, g.ldb), g.b_held, g.b_off);
                gemms.push_back(g);
            }
    }
};
static NoiseRecorder *g_noise = nullptr;  // set while a perturbative-noise product is recorded

template <typename S> struct Dumper : CallbackKernel {
    typedef DMRG<S, double, double> DMRGT;
    DMRGT *d = nullptr;
    Opts o;
    mutable vector<Region> regions;

    bool selected() const {
        if (o.dump_sweep != -1 && d->isweep != o.dump_sweep)
            return false;
        int site = d->me->center;
        if (o.dump_site == -2)
            return true;
        int want = o.dump_site == -1 ? d->me->n_sites / 2 - 1 : o.dump_site;
        return site == want;
    }
    string site_dir() const {
        stringstream ss;
        ss << o.out << "/sweep" << d->isweep << "_site" << d->me->center;
        return ss.str();
    }
    static void add_tensor(vector<Region> &r,
                           const shared_ptr<OperatorTensor<S, double>> &t) {
        if (t == nullptr)
            return;
        for (auto &kv : t->ops)
            if (kv.second != nullptr && kv.second->data != nullptr &&
                kv.second->total_memory != 0)
                r.push_back(Region{kv.second->data, kv.second->total_memory});
        if (t->get_type() == OperatorTensorTypes::Delayed) {
            auto dt = dynamic_pointer_cast<DelayedOperatorTensor<S, double>>(t);
            add_tensor(r, dt->lopt);
            add_tensor(r, dt->ropt);
        }
    }
    void collect_regions(const shared_ptr<EffectiveHamiltonian<S, double>> &h) const {
        regions.clear();
        add_tensor(regions, h->op->lopt);
        add_tensor(regions, h->op->ropt);
        sort(regions.begin(), regions.end(),
             [](const Region &a, const Region &b) { return a.p < b.p; });
        vector<Region> u;
        for (auto &r : regions)
            if (u.empty() || r.p != u.back().p)
                u.push_back(r);
            else
                u.back().n = max(u.back().n, r.n);
        regions = u;
    }
    // extent (in doubles) of an operand op(X) of shape rows x cols, leading dim ld
    static size_t extent(bool trans, int rows, int cols, int ld) {
        if (rows == 0 || cols == 0)
            return 0;
        return trans ? (size_t)(cols - 1) * ld + rows : (size_t)(rows - 1) * ld + cols;
    }
    long find_region(const double *p, size_t ext) const {
        auto it = upper_bound(regions.begin(), regions.end(), p,
                              [](const double *x, const Region &r) { return x < r.p; });
        if (it == regions.begin())
            return -1;
        --it;
        if (p >= it->p && p + ext <= it->p + it->n)
            return it - regions.begin();
        return -1;
    }

    void dump_pre(const shared_ptr<EffectiveHamiltonian<S, double>> &h) const {
        Writer w(site_dir());
        const size_t nket = h->ket->total_memory, nbra = h->bra->total_memory;
        collect_regions(h);
        h->precompute();
        auto seq = h->tf->opf->seq;
        auto b0 = seq->batch[0], b1 = seq->batch[1];
        if (!b0->acidxs.empty() || b0->c.size() != b0->gp.size() ||
            b1->c.size() != b1->gp.size() || b0->c.size() != b1->c.size())
            throw runtime_error("harness: recorded sequence is not a plain pair list");
        const size_t np = b0->c.size();
        const double *zero = (const double *)0;
        vector<int32_t> ta0(np), tb0(np), m0(np), n0(np), k0(np), lda0(np), ldb0(np);
        vector<int32_t> ta1(np), tb1(np), m1(np), n1(np), k1(np), lda1(np), ldb1(np), ldc1(np);
        vector<double> al0(np), be0(np), al1(np), be1(np);
        vector<uint64_t> a0(np), b0off(np), w0(np), a1(np), w1(np), c1(np);
        vector<int64_t> rb0(np), ra1(np);
        for (size_t i = 0; i < np; i++) {
            ta0[i] = b0->ta[i] != CblasNoTrans, tb0[i] = b0->tb[i] != CblasNoTrans;
            m0[i] = b0->m[i], n0[i] = b0->n[i], k0[i] = b0->k[i];
            lda0[i] = b0->lda[i], ldb0[i] = b0->ldb[i];
            al0[i] = b0->alpha[i], be0[i] = b0->beta[i];
            ta1[i] = b1->ta[i] != CblasNoTrans, tb1[i] = b1->tb[i] != CblasNoTrans;
            m1[i] = b1->m[i], n1[i] = b1->n[i], k1[i] = b1->k[i];
            lda1[i] = b1->lda[i], ldb1[i] = b1->ldb[i], ldc1[i] = b1->ldc[i];
            al1[i] = b1->alpha[i], be1[i] = b1->beta[i];
            if (b0->ldc[i] != b0->n[i] || ldb1[i] != n1[i] || tb1[i] != 0 || ta0[i] != 0)
                throw runtime_error("harness: unexpected work layout");
            a0[i] = (uint64_t)(b0->a[i] - zero);
            w0[i] = (uint64_t)(b0->c[i] - zero);
            w1[i] = (uint64_t)(b1->b[i] - zero);
            c1[i] = (uint64_t)(b1->c[i] - zero);
            if (w0[i] != w1[i])
                throw runtime_error("harness: work offsets differ within a pair");
            if (a0[i] + extent(false, m0[i], k0[i], lda0[i]) > nket)
                throw runtime_error("harness: psi operand out of range");
            if (c1[i] + extent(false, m1[i], n1[i], ldc1[i]) > nbra)
                throw runtime_error("harness: sigma operand out of range");
            rb0[i] = find_region(b0->b[i], extent(tb0[i], k0[i], n0[i], ldb0[i]));
            ra1[i] = find_region(b1->a[i], extent(ta1[i], m1[i], k1[i], lda1[i]));
            if (rb0[i] < 0 || ra1[i] < 0)
                throw runtime_error("harness: operator pointer outside the H_eff operators");
            regions[rb0[i]].used = regions[ra1[i]].used = true;
        }
        size_t blob = 0;
        for (auto &r : regions)
            if (r.used)
                r.blob_off = blob, blob += r.n;
        for (size_t i = 0; i < np; i++) {
            b0off[i] = regions[rb0[i]].blob_off + (b0->b[i] - regions[rb0[i]].p);
            a1[i] = regions[ra1[i]].blob_off + (b1->a[i] - regions[ra1[i]].p);
        }
        // sigma = H_eff * psi through the reference's own Tasked replay
        vector<double> psi(h->ket->data, h->ket->data + nket), sigma(nbra, 0.0);
        h->tf->operator()(GMatrix<double>(psi.data(), (MKL_INT)nket, 1),
                          GMatrix<double>(sigma.data(), (MKL_INT)nbra, 1), 1.0);
        size_t nflop = 0;
        for (size_t i = 0; i < np; i++)
            nflop += (size_t)m0[i] * n0[i] * k0[i] + (size_t)m1[i] * n1[i] * k1[i];
        h->post_precompute();
        w.scalar("n_pairs", (double)np);
        w.scalar("psi_size", (double)nket);
        w.scalar("sigma_size", (double)nbra);
        w.scalar("ops_size", (double)blob);
        w.scalar("mnk", (double)nflop);
        w.scalar("const_e", (double)d->me->mpo->const_e);
        w.scalar("isweep", d->isweep);
        w.scalar("site", d->me->center);
        w.scalar("n_sites", d->me->n_sites);
        w.scalar("forward", d->forward);
        w.scalar("conv_thrd", d->davidson_conv_thrds[min((size_t)d->isweep, d->davidson_conv_thrds.size() - 1)]);
        w.scalar("def_min", d->davidson_def_min_size);
        w.scalar("def_max", d->davidson_def_max_size);
        w.vec("ta0", ta0, "i4"), w.vec("tb0", tb0, "i4"), w.vec("m0", m0, "i4");
        w.vec("n0", n0, "i4"), w.vec("k0", k0, "i4"), w.vec("lda0", lda0, "i4");
        w.vec("ldb0", ldb0, "i4"), w.vec("alpha0", al0, "f8"), w.vec("beta0", be0, "f8");
        w.vec("ta1", ta1, "i4"), w.vec("tb1", tb1, "i4"), w.vec("m1", m1, "i4");
        w.vec("n1", n1, "i4"), w.vec("k1", k1, "i4"), w.vec("lda1", lda1, "i4");
        w.vec("ldb1", ldb1, "i4"), w.vec("ldc1", ldc1, "i4"), w.vec("alpha1", al1, "f8");
        w.vec("beta1", be1, "f8");
        w.vec("a0", a0, "u8"), w.vec("b0", b0off, "u8"), w.vec("w0", w0, "u8");
        w.vec("a1", a1, "u8"), w.vec("c1", c1, "u8");
        w.vec("psi", psi, "f8");
        w.vec("sigma", sigma, "f8");
        w.arr("diag", h->diag->data, h->diag->total_memory, "f8");
        // block structure of psi (= sigma for the ground state): quanta offsets and shapes
        {
            auto info = h->ket->info;
            vector<int32_t> rows(info->n), cols(info->n);
            vector<uint64_t> shifts(info->n);
            for (int i = 0; i < info->n; i++)
                rows[i] = info->n_states_bra[i], cols[i] = info->n_states_ket[i],
                shifts[i] = info->block_shifts[i];
            w.vec("psi_block_rows", rows, "i4");
            w.vec("psi_block_cols", cols, "i4");
            w.vec("psi_block_shift", shifts, "u8");
        }
        if (o.with_data) {
            vector<double> ops(blob);
            for (auto &r : regions)
                if (r.used)
                    memcpy(ops.data() + r.blob_off, r.p, sizeof(double) * r.n);
            w.vec("ops", ops, "f8");
        }
        w.man.flush();
    }
    // Quantum-number bookkeeping of the two-site wavefunction, as
    // MovingEnvironment::contract_two_dot builds it (moving_environment.hpp:3376-3387):
    // the input StateInfos, the two tensor products, the connection info of the
    // left one, a target-filtered product, and the wavefunction's block list.
    static void put_si(Writer &w, const string &name, const StateInfo<S> &si) {
        vector<uint64_t> q(si.n);
        vector<int32_t> n(si.n);
        for (int i = 0; i < si.n; i++)
            q[i] = si.quanta[i].data, n[i] = (int32_t)si.n_states[i];
        w.vec(name + "_q", q, "u8");
        w.vec(name + "_n", n, "i4");
    }
    void dump_quanta(const shared_ptr<EffectiveHamiltonian<S, double>> &h) const {
        Writer w(site_dir() + "/qn");
        auto mi = d->me->ket->info;
        const int c = d->me->center;
        mi->load_left_dims(c);
        mi->load_right_dims(c + 2);
        StateInfo<S> l = *mi->left_dims[c], ml = *mi->basis[c], mr = *mi->basis[c + 1],
                     r = *mi->right_dims[c + 2];
        StateInfo<S> ll = StateInfo<S>::tensor_product(l, ml, *mi->left_dims_fci[c + 1]);
        StateInfo<S> rr = StateInfo<S>::tensor_product(mr, r, *mi->right_dims_fci[c + 1]);
        StateInfo<S> lt = StateInfo<S>::tensor_product(l, ml, mi->target);
        auto lc = StateInfo<S>::get_connection_info(l, ml, ll);
        put_si(w, "l", l), put_si(w, "ml", ml), put_si(w, "mr", mr), put_si(w, "r", r);
        put_si(w, "lfci", *mi->left_dims_fci[c + 1]), put_si(w, "rfci", *mi->right_dims_fci[c + 1]);
        put_si(w, "ll", ll), put_si(w, "rr", rr), put_si(w, "lt", lt);
        vector<int32_t> acc(lc->acc_n_states.begin(), lc->acc_n_states.end()), ia, ib;
        for (auto &x : lc->ij_indices)
            ia.push_back((int32_t)x.first), ib.push_back((int32_t)x.second);
        w.vec("lc_acc", acc, "i4"), w.vec("lc_i", ia, "i4"), w.vec("lc_j", ib, "i4");
        auto info = h->ket->info;
        vector<uint64_t> q(info->n), sh(info->n);
        vector<int32_t> nb(info->n), nk(info->n);
        for (int i = 0; i < info->n; i++)
            q[i] = info->quanta[i].data, nb[i] = (int32_t)info->n_states_bra[i],
            nk[i] = (int32_t)info->n_states_ket[i], sh[i] = info->block_shifts[i];
        w.vec("wfn_q", q, "u8"), w.vec("wfn_rows", nb, "i4"), w.vec("wfn_cols", nk, "i4");
        w.vec("wfn_shift", sh, "u8");
        vector<uint64_t> dq{info->delta_quantum.data, mi->target.data};
        w.vec("dq_target", dq, "u8");
        w.scalar("is_wfn", info->is_wavefunction);
        w.scalar("total_memory", (double)h->ket->total_memory);
        w.scalar("su2", is_same<S, SU2>::value ? 1 : 0);
        dump_wfn_cinfo(w, h);
        if (o.effprob) {
            // the reference's own export of this H_eff (EffectiveHamiltonian::
            // save_eff_problem, src/dmrg/effective_hamiltonian.hpp:254-261,
            // writing the EFFPROB1 format of src/core/effective_problem.hpp),
            // moved next to the connection infos above; sweeps alternate
            // direction starting forward
            const bool fw = d->isweep % 2 == 0;
            h->save_eff_problem(c, fw);
            const string src = frame_<double>()->save_dir + "/EFF-PROB." + (fw ? "FORW." : "BACKW.") +
                               Parsing::to_string(c);
            if (rename(src.c_str(), (site_dir() + "/qn/effprob.bin").c_str()) != 0)
                throw runtime_error("harness: cannot move " + src);
            w.scalar("effprob_isite", c), w.scalar("effprob_forward", fw ? 1 : 0);
        }
        w.man.flush();
        lc = nullptr;
        lt.deallocate(), rr.deallocate(), ll.deallocate();
    }
    // The H_eff's wavefunction connection infos (ConnectionInfo::initialize_wfn,
    // src/core/sparse_matrix.hpp:163-292, built in the EffectiveHamiltonian
    // constructor, src/dmrg/effective_hamiltonian.hpp:208-216) with their
    // inputs: the left/right operator infos, ket/bra infos and labels.
    static void put_op_infos(Writer &w, const string &name,
                             const vector<pair<S, shared_ptr<SparseMatrixInfo<S>>>> &infos) {
        vector<uint64_t> dq, q;
        vector<int32_t> ferm, start;
        for (auto &p : infos) {
            dq.push_back(p.first.data);
            ferm.push_back(p.second->is_fermion ? 1 : 0);
            start.push_back((int32_t)q.size());
            for (int i = 0; i < p.second->n; i++)
                q.push_back(p.second->quanta[i].data);
        }
        start.push_back((int32_t)q.size());
        w.vec(name + "_dq", dq, "u8"), w.vec(name + "_ferm", ferm, "i4");
        w.vec(name + "_start", start, "i4"), w.vec(name + "_q", q, "u8");
    }
    void dump_wfn_cinfo(Writer &w, const shared_ptr<EffectiveHamiltonian<S, double>> &h) const {
        put_op_infos(w, "lop", h->left_op_infos);
        put_op_infos(w, "rop", h->right_op_infos);
        vector<uint64_t> bq(h->bra->info->n);
        for (int i = 0; i < h->bra->info->n; i++)
            bq[i] = h->bra->info->quanta[i].data;
        w.vec("bra_q", bq, "u8");
        vector<uint64_t> lab{h->ket->info->delta_quantum.data, h->bra->info->delta_quantum.data};
        vector<uint64_t> opq, cq, cstride;
        vector<int32_t> cn, cidx, cia, cib, cic, cstart, cqstart;
        vector<double> cf;
        for (size_t i = 0; i < h->wfn_infos.size(); i++) {
            auto ci = h->wfn_infos[i];
            if (ci == nullptr)
                continue;
            opq.push_back(h->operator_quanta[i].data);
            for (int t = 0; t < 5; t++)
                cn.push_back(ci->n[t]);
            cqstart.push_back((int32_t)cq.size());
            for (int k = 0; k < ci->n[4]; k++)
                cq.push_back(ci->quanta[k].data), cidx.push_back((int32_t)ci->idx[k]);
            cstart.push_back((int32_t)cstride.size());
            for (int j = 0; j < ci->nc; j++) {
                cstride.push_back(ci->stride[j]), cf.push_back(ci->factor[j]);
                cia.push_back((int32_t)ci->ia[j]), cib.push_back((int32_t)ci->ib[j]);
                cic.push_back((int32_t)ci->ic[j]);
            }
        }
        cqstart.push_back((int32_t)cq.size()), cstart.push_back((int32_t)cstride.size());
        w.vec("cdq_vdq", lab, "u8"), w.vec("ci_opdq", opq, "u8"), w.vec("ci_n", cn, "i4");
        w.vec("ci_q", cq, "u8"), w.vec("ci_qstart", cqstart, "i4"), w.vec("ci_idx", cidx, "i4");
        w.vec("ci_start", cstart, "i4"), w.vec("ci_stride", cstride, "u8"), w.vec("ci_factor", cf, "f8");
        w.vec("ci_ia", cia, "i4"), w.vec("ci_ib", cib, "i4"), w.vec("ci_ic", cic, "i4");
    }
    void dump_post(const shared_ptr<EffectiveHamiltonian<S, double>> &h) const {
        Writer w(site_dir() + "/post");
        const size_t nket = h->ket->total_memory, nbra = h->bra->total_memory;
        vector<double> psi(h->ket->data, h->ket->data + nket), sigma(nbra, 0.0);
        h->precompute();
        h->tf->operator()(GMatrix<double>(psi.data(), (MKL_INT)nket, 1),
                          GMatrix<double>(sigma.data(), (MKL_INT)nbra, 1), 1.0);
        h->post_precompute();
        double e = 0, nn = 0;
        for (size_t i = 0; i < nket; i++)
            e += psi[i] * sigma[i], nn += psi[i] * psi[i];
        w.scalar("energy", e / nn + (double)d->me->mpo->const_e);
        w.scalar("norm2", nn);
        w.vec("psi", psi, "f8");
        w.man.flush();
        dump_truncation(h);
    }
    // The perturbative-noise product of the converged ket, requested the way
    // DMRG::two_dot_eigs_and_perturb does (src/dmrg/sweep_algorithm.hpp:1257-1260) with
    // NoiseTypes::ReducedPerturbative (or the NoiseTypes value --noise-product
    // gives, e.g. 4 = Perturbative, 76 = ReducedPerturbativeLowMem).  Written: the recorded GEMMs
    // (c += alpha op(a) op(b); g_akind/g_bkind 0 = ket, 1 = operator blob; g_c an
    // offset into the perturbed group), the operator blob they read, the ket
    // ("psi"), the reference's perturbed-wavefunction group ("sigma") and the
    // group's block layout.
    void dump_noise(const shared_ptr<EffectiveHamiltonian<S, double>> &h) const {
        const bool forward = d->isweep % 2 == 0;  // solve() starts forward and alternates
        const int isite = d->me->center;
        collect_regions(h);
        auto seq = h->tf->opf->seq;
        if (!seq->batch[0]->c.empty() || !seq->batch[1]->c.empty())
            throw runtime_error("harness: GEMM sequence not empty before the noise product");
        NoiseRecorder R;
        R.ket = h->ket->data, R.nket = h->ket->total_memory;
        R.known = [this](const double *p, size_t ext) { return find_region(p, ext) >= 0; };
        g_noise = &R;
        const NoiseTypes nt = o.noise == 1 ? NoiseTypes::ReducedPerturbative : (NoiseTypes)o.noise;
        if (!(nt & NoiseTypes::Perturbative))
            throw runtime_error("harness: --noise-product needs a perturbative noise type");
        auto pket = h->perturbative_noise(forward, isite, isite + 1, FuseTypes::FuseLR,
                                          d->me->ket->info, nt);
        g_noise = nullptr;
        const double *vbase = pket->data;
        const size_t nsig = pket->total_memory;
        // blob: the H_eff operator regions the GEMMs read, then the held copies
        for (auto &r : regions)
            r.used = false;
        auto in_ket = [&](const double *p, int held) { return held < 0 && p >= R.ket && p < R.ket + R.nket; };
        for (auto &g : R.gemms)
            for (auto pr : {make_pair(g.a, g.a_held), make_pair(g.b, g.b_held)})
                if (pr.second < 0 && !in_ket(pr.first, pr.second))
                    regions[find_region(pr.first, 1)].used = true;
        size_t blob = 0;
        for (auto &r : regions)
            if (r.used)
                r.blob_off = blob, blob += r.n;
        vector<size_t> held_off(R.held.size());
        for (size_t q = 0; q < R.held.size(); q++)
            held_off[q] = blob, blob += R.held[q].size();
        vector<double> ops(blob);
        for (auto &r : regions)
            if (r.used)
                memcpy(ops.data() + r.blob_off, r.p, sizeof(double) * r.n);
        for (size_t q = 0; q < R.held.size(); q++)
            memcpy(ops.data() + held_off[q], R.held[q].data(), sizeof(double) * R.held[q].size());
        const size_t ng = R.gemms.size();
        vector<int32_t> ta(ng), tb(ng), m(ng), n(ng), k(ng), lda(ng), ldb(ng), ldc(ng), ak(ng), bk(ng);
        vector<double> al(ng), be(ng);
        vector<uint64_t> ga(ng), gb(ng), gc(ng);
        auto where = [&](const double *p, int held, size_t hoff, int32_t &kind) -> uint64_t {
            if (in_ket(p, held))
                return kind = 0, (uint64_t)(p - R.ket);
            kind = 1;
            if (held >= 0)
                return held_off[held] + hoff;
            const long ri = find_region(p, 1);
            return regions[ri].blob_off + (size_t)(p - regions[ri].p);
        };
        for (size_t q = 0; q < ng; q++) {
            const auto &g = R.gemms[q];
            if (g.c < vbase || g.c >= vbase + nsig)
                throw runtime_error("harness: noise GEMM output outside the perturbed group");
            ta[q] = g.ta, tb[q] = g.tb, m[q] = g.m, n[q] = g.n, k[q] = g.k;
            lda[q] = g.lda, ldb[q] = g.ldb, ldc[q] = g.ldc, al[q] = g.alpha, be[q] = g.beta;
            ga[q] = where(g.a, g.a_held, g.a_off, ak[q]);
            gb[q] = where(g.b, g.b_held, g.b_off, bk[q]);
            gc[q] = (uint64_t)(g.c - vbase);
        }
        vector<double> psi(R.ket, R.ket + R.nket), sigma(vbase, vbase + nsig);
        vector<int32_t> vrows, vcols, vidx;
        vector<uint64_t> vq, voff;
        for (int j = 0; j < pket->n; j++) {
            const auto &info = pket->infos[j];
            vq.push_back(info->delta_quantum.data);
            for (int b = 0; b < info->n; b++) {
                vrows.push_back(info->n_states_bra[b]), vcols.push_back(info->n_states_ket[b]);
                voff.push_back(pket->offsets[j] + info->block_shifts[b]), vidx.push_back(j);
            }
        }
        Writer w(site_dir() + "/noise");
        w.scalar("n_gemms", (double)ng), w.scalar("n_held", (double)R.held.size());
        w.scalar("forward", forward), w.scalar("n_vectors", pket->n), w.scalar("noise_type", (double)(uint16_t)nt);
        w.scalar("psi_size", (double)R.nket), w.scalar("sigma_size", (double)nsig);
        w.scalar("ops_size", (double)blob);
        w.vec("g_ta", ta, "i4"), w.vec("g_tb", tb, "i4"), w.vec("g_m", m, "i4"), w.vec("g_n", n, "i4");
        w.vec("g_k", k, "i4"), w.vec("g_lda", lda, "i4"), w.vec("g_ldb", ldb, "i4"), w.vec("g_ldc", ldc, "i4");
        w.vec("g_akind", ak, "i4"), w.vec("g_bkind", bk, "i4"), w.vec("g_alpha", al, "f8");
        w.vec("g_beta", be, "f8"), w.vec("g_a", ga, "u8"), w.vec("g_b", gb, "u8"), w.vec("g_c", gc, "u8");
        w.vec("psi", psi, "f8"), w.vec("ops", ops, "f8"), w.vec("sigma", sigma, "f8");
        w.vec("vec_q", vq, "u8"), w.vec("blk_rows", vrows, "i4"), w.vec("blk_cols", vcols, "i4");
        w.vec("blk_off", voff, "u8"), w.vec("blk_vec", vidx, "i4");
        w.man.flush();
        pket->deallocate();
        pket->deallocate_infos();
    }
    // Density matrix of the converged psi, its spectrum, and the reference's
    // truncation/split (MovingEnvironment::density_matrix / split_density_matrix,
    // src/dmrg/moving_environment.hpp:3554-3580, 4250-4345) on copies.
    void dump_truncation(const shared_ptr<EffectiveHamiltonian<S, double>> &h) const {
        Writer w(site_dir() + "/truncation");
        const bool trace_right = d->isweep % 2 == 0;  // solve() starts forward and alternates
        auto vmem = make_shared<VectorAllocator<double>>();
        auto psi = make_shared<SparseMatrix<S, double>>(vmem);
        psi->allocate(h->ket->info);
        memcpy(psi->data, h->ket->data, sizeof(double) * psi->total_memory);
        const S vacuum = d->me->ket->info->vacuum;
        auto dm = MovingEnvironment<S, double, double>::density_matrix(vacuum, psi, trace_right, 0.0,
                                                                       NoiseTypes::None);
        // psi block -> dm block (the mapping trans_product uses)
        vector<int32_t> psi_dm(psi->info->n), psi_rows(psi->info->n), psi_cols(psi->info->n);
        vector<uint64_t> psi_off(psi->info->n);
        for (int ia = 0; ia < psi->info->n; ia++) {
            S q = trace_right ? psi->info->quanta[ia].get_bra(psi->info->delta_quantum)
                              : -psi->info->quanta[ia].get_ket();
            psi_dm[ia] = dm->info->find_state(q);
            psi_rows[ia] = psi->info->n_states_bra[ia], psi_cols[ia] = psi->info->n_states_ket[ia];
            psi_off[ia] = psi->info->block_shifts[ia];
        }
        vector<int32_t> dm_dim(dm->info->n);
        vector<uint64_t> dm_off(dm->info->n);
        vector<double> eig;
        for (int ib = 0; ib < dm->info->n; ib++) {
            dm_dim[ib] = dm->info->n_states_bra[ib], dm_off[ib] = dm->info->block_shifts[ib];
            GMatrix<double> blk = (*dm)[ib];
            vector<double> a(blk.data, blk.data + (size_t)blk.m * blk.n), ww(blk.m);
            GMatrixFunctions<double>::eigs(GMatrix<double>(a.data(), blk.m, blk.n),
                                           GDiagonalMatrix<double>(ww.data(), blk.m));
            eig.insert(eig.end(), ww.begin(), ww.end());
        }
        vector<double> rho(dm->data, dm->data + dm->total_memory);
        shared_ptr<SparseMatrix<S, double>> left, right;
        vector<double> spectra;
        const int M = (int)d->bond_dims[min((size_t)d->isweep, d->bond_dims.size() - 1)];
        double err = MovingEnvironment<S, double, double>::split_density_matrix(
            dm, psi, M, trace_right, true, left, right, d->cutoff, false, spectra, d->trunc_type);
        auto blocks = [&](const shared_ptr<SparseMatrix<S, double>> &m, const char *tag, bool is_left) {
            vector<int32_t> rows(m->info->n), cols(m->info->n), link(m->info->n);
            vector<uint64_t> off(m->info->n);
            for (int i = 0; i < m->info->n; i++) {
                rows[i] = m->info->n_states_bra[i], cols[i] = m->info->n_states_ket[i];
                off[i] = m->info->block_shifts[i];
                // link: dm block (rotation side) or psi block (wavefunction side)
                // (rotation blocks carry their dm block's quantum,
                // rotation_matrix_info_from_density_matrix)
                if (is_left == trace_right)
                    link[i] = dm->info->find_state(m->info->quanta[i]);
                else
                    link[i] = psi->info->find_state(m->info->quanta[i]);
            }
            string t(tag);
            w.vec(t + "_rows", rows, "i4"), w.vec(t + "_cols", cols, "i4");
            w.vec(t + "_off", off, "u8"), w.vec(t + "_link", link, "i4");
            w.arr(t + "_data", m->data, m->total_memory, "f8");
        };
        w.scalar("trace_right", trace_right);
        w.scalar("bond_dim", M);
        w.scalar("cutoff", d->cutoff);
        w.scalar("error", err);
        w.vec("psi_dm", psi_dm, "i4"), w.vec("psi_rows", psi_rows, "i4"), w.vec("psi_cols", psi_cols, "i4");
        w.vec("psi_off", psi_off, "u8");
        w.vec("dm_dim", dm_dim, "i4"), w.vec("dm_off", dm_off, "u8");
        w.vec("dm_eig", eig, "f8"), w.vec("rho", rho, "f8");
        blocks(left, "left", true);
        blocks(right, "right", false);
        w.man.flush();
        right->deallocate(), left->deallocate(), dm->deallocate();  // stack order
        right->info->deallocate(), left->info->deallocate(), dm->info->deallocate();
        psi->deallocate();
    }
    // the next operator rotation after a dumped site is recorded too
    mutable bool want_rotation = false;
    mutable bool want_blocking = false;  // the next left/right_contract is recorded
    mutable string rot_dir, blk_dir;
    void compute(const string &name, int iprint) const override {
        if (d == nullptr || d->current_eff_ham == nullptr || !selected())
            return;
        if (name == "DMRG::sweep::iter.eff_ham") {
            dump_pre(d->current_eff_ham);
            dump_quanta(d->current_eff_ham);
        }
        else if (name == "DMRG::sweep::iter.eff_ham.end") {
            dump_post(d->current_eff_ham);
            if (o.noise != 0)
                dump_noise(d->current_eff_ham);
            want_rotation = true;
            want_blocking = true;
            rot_dir = site_dir() + "/rotation";
            blk_dir = site_dir() + "/blocking";
        }
    }
};

// Blocking recorder.  TensorFunctions::left_contract / right_contract
// (src/core/tensor_functions.hpp:2842-2986) run unchanged; while one is being
// recorded, the OperatorFunctions calls they make are logged at block level,
// restating the block loops of OperatorFunctions::iadd
// (src/core/operator_functions.hpp:135-170: a_blk = a_blk + f op(b_blk)) and
// OperatorFunctions::tensor_product (operator_functions.hpp:672-710, through
// GMatrixFunctions::tensor_product, src/core/matrix_functions.hpp:1269-1400:
// c[stride + (i bm' + k) c.n + j bn' + l] += f A'(i,j) B'(k,l), A' = op(a_blk),
// B' = op(b_blk)).  Operands live in four blobs: the enlarged block's inputs
// (env ops and site ops), intermediates (sums built by iadd) and the outputs.
struct BlockRecorder {
    std::mutex mu;
    map<const double *, pair<int, size_t>> where;  // data pointer -> (blob, offset)
    vector<double> env, site;
    size_t tmp_size = 0;
    map<const double *, size_t> tmp_open;          // live intermediates
    map<const double *, size_t> out_off;           // output matrices (packed after)
    // records
    vector<int32_t> ia_m, ia_n, ia_conj;           // iadd: dst block m x n, src transposed
    vector<uint64_t> ia_dst, ia_src;
    vector<int32_t> ia_src_blob;
    vector<double> ia_f;
    vector<int32_t> kr_am, kr_an, kr_ca, kr_bm, kr_bn, kr_cb, kr_cn, kr_ablob, kr_bblob;
    vector<uint64_t> kr_a, kr_b, kr_c;
    vector<double> kr_f;
    size_t out_size = 0;
    vector<pair<const double *, size_t>> out_list;  // (data, total_memory) in order
    size_t pack(vector<double> &blob, const double *p, size_t n) {
        size_t o = blob.size();
        blob.insert(blob.end(), p, p + n);
        return o;
    }
    // where an operand's data lives (an intermediate is opened by its first iadd)
    pair<int, size_t> locate(const double *p) {
        auto it = where.find(p);
        if (it != where.end())
            return it->second;
        auto t = tmp_open.find(p);
        if (t != tmp_open.end())
            return make_pair(2, t->second);
        return make_pair(-1, (size_t)0);
    }
};
static BlockRecorder *g_blk = nullptr;  // set while a contraction is recorded

// Fast-expectation recorder (TensorFunctions::tensor_product_expectation,
// src/core/tensor_functions.hpp:1701-1877, the algorithm Expect uses for PDM
// MPOs).  For every unique left operator a it builds a partial
// b = <bra| a |ket> (OperatorFunctions::tensor_left_partial_expectation,
// src/core/operator_functions.hpp:354-410: per connected block,
// work = op(a) ket, then b += bra^T work or work^T bra, through
// BatchGEMMSeq::left_partial_rotate, src/core/batch_gemm.hpp:904-922), and
// each expectation is a sum of factor * dot(partial, right operator).  The
// block loop is restated here and every block written as a GEMM pair of the
// H_eff format with the left operator as the pair's left GEMM0 operand
// ("psi"), ket and bra in the operator blob ("ops") and the partials as the
// output ("sigma"); a partial whose blocks come out transposed (conj bits
// differ) is stored block-transposed.
struct NpdmRecorder {
    std::mutex mu;
    int calls = 0, want = -1;
    bool active = false;
    string out;
    const double *ket = nullptr, *bra = nullptr;
    size_t nket = 0, nbra = 0;
    map<const double *, size_t> lop_off;  // left operator data -> offset in lops
    vector<double> lops;
    struct Part {
        size_t off;
        bool trans;
        vector<int32_t> rows, cols;
        vector<uint64_t> boff;  // block offsets within the partial
    };
    map<tuple<int, uint64_t, uint64_t, const double *>, int> part_key;  // (conj, rdq, opdq, a data)
    vector<Part> parts;
    size_t sig = 0;
    vector<double> ref;  // the reference's partials, in the storage layout
    vector<int32_t> tb0, m0, n0, k0, lda0, ldb0, ta1, m1, n1, k1, lda1, ldc1;
    vector<double> al0, al1;
    vector<uint64_t> a0, b0, a1, c1;
};
static NpdmRecorder *g_npdm = nullptr;  // set while a PDM expectation sweep runs

template <typename S> struct RecordingOpf : OperatorFunctions<S, double> {
    typedef OperatorFunctions<S, double> OPF;
    explicit RecordingOpf(const shared_ptr<CG<S>> &cg) : OPF(cg) {}
    shared_ptr<OPF> copy() const override {
        shared_ptr<OPF> p = make_shared<RecordingOpf>(this->cg);
        p->seq = this->seq->copy();
        return p;
    }
    void iadd(const shared_ptr<SparseMatrix<S, double>> &a, const shared_ptr<SparseMatrix<S, double>> &b,
              double scale = 1.0, bool conj = false) const override {
        BlockRecorder *R = g_blk;
        if (R != nullptr && abs(b->factor * scale) >= TINY) {
            lock_guard<std::mutex> lk(R->mu);
            if (a->factor != 1.0)
                throw runtime_error("blocking recorder: iadd into a scaled matrix");
            // the destination is an intermediate: open it at its first use
            size_t dst_base;
            auto t = R->tmp_open.find(a->data);
            if (t == R->tmp_open.end()) {
                dst_base = R->tmp_size;
                R->tmp_open[a->data] = dst_base;
                R->tmp_size += a->total_memory;
            } else
                dst_base = t->second;
            pair<int, size_t> src = R->locate(b->data);
            if (src.first < 0)
                throw runtime_error("blocking recorder: iadd source not found");
            S bdq = b->info->delta_quantum;
            for (int ia = 0, ib; ia < a->info->n; ia++) {
                S bra = a->info->quanta[ia].get_bra(a->info->delta_quantum);
                S ket = a->info->quanta[ia].get_ket();
                S bq = conj ? bdq.combine(ket, bra) : bdq.combine(bra, ket);
                if (bq == S(S::invalid) || (ib = b->info->find_state(bq)) == -1)
                    continue;
                double f = scale * b->factor;
                if (conj)
                    f *= this->cg->transpose_cg(bdq, bra, ket);
                GMatrix<double> ma = (*a)[ia], mb = (*b)[ib];
                R->ia_m.push_back(ma.m), R->ia_n.push_back(ma.n), R->ia_conj.push_back(conj ? 1 : 0);
                R->ia_dst.push_back(dst_base + (ma.data - a->data));
                R->ia_src_blob.push_back(src.first);
                R->ia_src.push_back(src.second + (mb.data - b->data));
                R->ia_f.push_back(f);
            }
        }
        OPF::iadd(a, b, scale, conj);
    }
    void tensor_product(uint8_t conj, const shared_ptr<SparseMatrix<S, double>> &a,
                        const shared_ptr<SparseMatrix<S, double>> &b,
                        const shared_ptr<SparseMatrix<S, double>> &c, double scale = 1.0) const override {
        BlockRecorder *R = g_blk;
        if (R != nullptr) {
            lock_guard<std::mutex> lk(R->mu);
            const double sc = scale * a->factor * b->factor;
            if (abs(sc) >= TINY && a->data != nullptr && b->data != nullptr && c->data != nullptr) {
                if (c->factor != 1.0)
                    throw runtime_error("blocking recorder: scaled output");
                pair<int, size_t> la = R->locate(a->data), lb = R->locate(b->data);
                if (la.first < 0 || lb.first < 0)
                    throw runtime_error("blocking recorder: operand not found");
                auto oc = R->out_off.find(c->data);
                size_t cbase;
                if (oc == R->out_off.end()) {
                    cbase = R->out_size;
                    R->out_off[c->data] = cbase;
                    R->out_size += c->total_memory;
                    R->out_list.push_back(make_pair((const double *)c->data, (size_t)c->total_memory));
                } else
                    cbase = oc->second;
                S adq = a->info->delta_quantum, bdq = b->info->delta_quantum, cdq = c->info->delta_quantum;
                auto cinfo = c->info->cinfo;
                S abdq = cdq.combine((conj & 1) ? -adq : adq, (conj & 2) ? bdq : -bdq);
                int ik = (int)(lower_bound(cinfo->quanta + cinfo->n[conj], cinfo->quanta + cinfo->n[conj + 1],
                                           abdq) - cinfo->quanta);
                int ixa = cinfo->idx[ik];
                int ixb = ik == cinfo->n[4] - 1 ? cinfo->nc : cinfo->idx[ik + 1];
                for (int il = ixa; il < ixb; il++) {
                    int ia = cinfo->ia[il], ib = cinfo->ib[il], ic = cinfo->ic[il];
                    GMatrix<double> ma = (*a)[ia], mb = (*b)[ib], mc = (*c)[ic];
                    R->kr_am.push_back(ma.m), R->kr_an.push_back(ma.n), R->kr_ca.push_back(conj & 1);
                    R->kr_bm.push_back(mb.m), R->kr_bn.push_back(mb.n), R->kr_cb.push_back((conj & 2) >> 1);
                    R->kr_cn.push_back(mc.n);
                    R->kr_ablob.push_back(la.first), R->kr_bblob.push_back(lb.first);
                    R->kr_a.push_back(la.second + (ma.data - a->data));
                    R->kr_b.push_back(lb.second + (mb.data - b->data));
                    R->kr_c.push_back(cbase + (mc.data - c->data) + cinfo->stride[il]);
                    R->kr_f.push_back(sc * cinfo->factor[il]);
                }
                // an intermediate is consumed by one product; its memory may be reused
                if (la.first == 2)
                    R->tmp_open.erase(a->data);
                if (lb.first == 2)
                    R->tmp_open.erase(b->data);
            }
        }
        OPF::tensor_product(conj, a, b, c, scale);
    }
    // the GEMMs of a perturbative-noise product, read right after each call adds them
    void tensor_product_multiply(uint8_t conj, const shared_ptr<SparseMatrix<S, double>> &a,
                                 const shared_ptr<SparseMatrix<S, double>> &b,
                                 const shared_ptr<SparseMatrix<S, double>> &c,
                                 const shared_ptr<SparseMatrix<S, double>> &v, S opdq,
                                 double scale = 1.0, TraceTypes tt = TraceTypes::None) const override {
        OPF::tensor_product_multiply(conj, a, b, c, v, opdq, scale, tt);
        if (g_noise != nullptr)
            g_noise->take(*this->seq->batch[1], {{a->data, a->total_memory}, {b->data, b->total_memory}});
    }
    void three_tensor_product_multiply(uint8_t conj, const shared_ptr<SparseMatrix<S, double>> &a,
                                       const shared_ptr<SparseMatrix<S, double>> &b,
                                       const shared_ptr<SparseMatrix<S, double>> &c,
                                       const shared_ptr<SparseMatrix<S, double>> &v, uint8_t dconj,
                                       const shared_ptr<SparseMatrix<S, double>> &da,
                                       const shared_ptr<SparseMatrix<S, double>> &db, bool dleft, S opdq,
                                       double scale = 1.0, TraceTypes tt = TraceTypes::None) const override {
        OPF::three_tensor_product_multiply(conj, a, b, c, v, dconj, da, db, dleft, opdq, scale, tt);
        if (g_noise != nullptr)
            g_noise->take(*this->seq->batch[1], {{a->data, a->total_memory}, {b->data, b->total_memory},
                                                 {da->data, da->total_memory}, {db->data, db->total_memory}});
    }
    // one partial of the fast expectation (see NpdmRecorder): the reference
    // computes it, then its blocks are recorded as GEMM pairs
    void tensor_left_partial_expectation(uint8_t conj, const shared_ptr<SparseMatrix<S, double>> &a,
                                         const shared_ptr<SparseMatrix<S, double>> &b,
                                         const shared_ptr<SparseMatrix<S, double>> &c,
                                         const shared_ptr<SparseMatrix<S, double>> &v, S opdq,
                                         double scale = 1.0) const override {
        OPF::tensor_left_partial_expectation(conj, a, b, c, v, opdq, scale);
        NpdmRecorder *R = g_npdm;
        if (R == nullptr || !R->active)
            return;
        lock_guard<std::mutex> lk(R->mu);
        if (c->data != R->ket || v->data != R->bra)
            throw runtime_error("npdm recorder: partial of another ket or bra");
        const bool ca = conj & 1, cc = (conj & 2) >> 1;
        // the partial (sigma role), its blocks and the reference's values
        const int pid = (int)R->parts.size();
        NpdmRecorder::Part P;
        P.off = R->sig, P.trans = ca != cc;
        for (int ib = 0; ib < b->info->n; ib++) {
            P.rows.push_back((int32_t)b->info->n_states_bra[ib]);
            P.cols.push_back((int32_t)b->info->n_states_ket[ib]);
            P.boff.push_back(b->info->block_shifts[ib]);
        }
        R->ref.resize(R->sig + b->total_memory, 0.0);
        for (int ib = 0; ib < b->info->n; ib++) {
            const double *src = b->data + P.boff[ib];
            double *dst = R->ref.data() + P.off + P.boff[ib];
            const int rr = P.rows[ib], cl = P.cols[ib];
            for (int i = 0; i < rr; i++)
                for (int j = 0; j < cl; j++)
                    (P.trans ? dst[(size_t)j * rr + i] : dst[(size_t)i * cl + j]) = src[(size_t)i * cl + j];
        }
        R->sig += b->total_memory;
        R->parts.push_back(P);
        R->part_key[make_tuple((int)conj, (uint64_t)b->info->delta_quantum.data, (uint64_t)opdq.data,
                               (const double *)a->data)] = pid;
        // restating the block loop (operator_functions.hpp:364-394); FL is real,
        // so the conjugations there are the identity
        const double s0 = scale * a->factor * v->factor * c->factor;
        if (abs(s0) < TINY)
            return;
        if (R->lop_off.count(a->data) == 0) {
            R->lop_off[a->data] = R->lops.size();
            R->lops.insert(R->lops.end(), a->data, a->data + a->total_memory);
        }
        const size_t abase = R->lop_off[a->data];
        const size_t vbase = R->bra == R->ket ? 0 : R->nket;
        S adq = a->info->delta_quantum, bdq = b->info->delta_quantum;
        auto cinfo = c->info->cinfo;
        S abdq = opdq.combine((conj & 1) ? -adq : adq, (conj & 2) ? bdq : -bdq);
        const int ik = (int)(lower_bound(cinfo->quanta + cinfo->n[conj], cinfo->quanta + cinfo->n[conj + 1], abdq) -
                             cinfo->quanta);
        const int ixa = cinfo->idx[ik], ixb = ik == cinfo->n[4] - 1 ? cinfo->nc : cinfo->idx[ik + 1];
        for (int il = ixa; il < ixb; il++) {
            const int ia = cinfo->ia[il], ib = cinfo->ib[il], ic = cinfo->ic[il], iv = (int)cinfo->stride[il];
            const double sc = s0 * cinfo->factor[il];
            GMatrix<double> A = (*a)[ia], C = (*b)[ib], V = (*v)[iv], K = (*c)[ic];
            const uint64_t offA = abase + (uint64_t)(A.data - a->data);
            const uint64_t offK = (uint64_t)(K.data - R->ket), offV = vbase + (uint64_t)(V.data - R->bra);
            const uint64_t offC = P.off + (uint64_t)(C.data - b->data);
            // W = A op2 with op2 = ket (no ca) or bra (ca); out (+)= op1^T W with op1 the other one
            const GMatrix<double> &X = ca ? V : K, &Y = ca ? K : V;
            if (A.n != X.m || Y.m != A.m)
                throw runtime_error("npdm recorder: block shapes do not chain");
            const bool out_t = ca != cc;  // block written transposed
            const int orow = out_t ? C.n : C.m, ocol = out_t ? C.m : C.n;
            if (orow != Y.n || ocol != X.n)
                throw runtime_error("npdm recorder: partial block shape");
            R->tb0.push_back(0), R->m0.push_back(A.m), R->k0.push_back(A.n), R->n0.push_back(X.n);
            R->lda0.push_back(A.n), R->ldb0.push_back(X.n), R->a0.push_back(offA);
            R->b0.push_back(ca ? offV : offK);
            R->ta1.push_back(1), R->m1.push_back(Y.n), R->k1.push_back(Y.m), R->n1.push_back(X.n);
            R->lda1.push_back(Y.n), R->a1.push_back(ca ? offK : offV);
            R->ldc1.push_back(ocol), R->c1.push_back(offC);
            R->al0.push_back(1.0), R->al1.push_back(sc);
        }
    }
};

// Operator rotation recorder: TensorFunctions::left_rotate / right_rotate
// (src/core/tensor_functions.hpp:2365-2403) run unchanged; when a rotation is
// requested, its per-block GEMM pairs are written in the same pair format as
// H_eff*psi, restating the block loop of OperatorFunctions::tensor_rotate
// (src/core/operator_functions.hpp:175-211) and the GEMM order of
// GMatrixFunctions::rotate (src/core/matrix_functions.hpp:998-1009):
//   work = a * op(ket);  c += scale * op(bra) * work.
// "psi" is the packed input operator data, "ops" the MPS tensor (bra, ket),
// "sigma" the packed rotated operators (the reference's result).
template <typename S> struct RecordingTF : TensorFunctions<S, double> {
    typedef TensorFunctions<S, double> TF;
    const Dumper<S> *dumper = nullptr;
    RecordingTF(const shared_ptr<OperatorFunctions<S, double>> &opf, const Dumper<S> *dp)
        : TF(opf), dumper(dp) {}
    shared_ptr<TF> copy() const override {
        return make_shared<RecordingTF>(this->opf->copy(), dumper);
    }
    void left_contract(const shared_ptr<OperatorTensor<S, double>> &a,
                       const shared_ptr<OperatorTensor<S, double>> &b,
                       shared_ptr<OperatorTensor<S, double>> &c,
                       const shared_ptr<Symbolic<S>> &cexprs = nullptr,
                       OpNamesSet delayed = OpNamesSet()) const override {
        if (!begin_blocking(a, b))
            return TF::left_contract(a, b, c, cexprs, delayed);
        TF::left_contract(a, b, c, cexprs, delayed);
        end_blocking(false);
    }
    void right_contract(const shared_ptr<OperatorTensor<S, double>> &a,
                        const shared_ptr<OperatorTensor<S, double>> &b,
                        shared_ptr<OperatorTensor<S, double>> &c,
                        const shared_ptr<Symbolic<S>> &cexprs = nullptr,
                        OpNamesSet delayed = OpNamesSet()) const override {
        if (!begin_blocking(a, b))
            return TF::right_contract(a, b, c, cexprs, delayed);
        TF::right_contract(a, b, c, cexprs, delayed);
        end_blocking(true);
    }
    mutable shared_ptr<BlockRecorder> blk;
    bool begin_blocking(const shared_ptr<OperatorTensor<S, double>> &a,
                        const shared_ptr<OperatorTensor<S, double>> &b) const {
        if (dumper == nullptr || !dumper->want_blocking || a == nullptr)
            return false;
        dumper->want_blocking = false;
        blk = make_shared<BlockRecorder>();
        for (auto &p : a->ops)
            if (p.second->data != nullptr && blk->where.count(p.second->data) == 0)
                blk->where[p.second->data] =
                    make_pair(0, blk->pack(blk->env, p.second->data, p.second->total_memory));
        for (auto &p : b->ops)
            if (p.second->data != nullptr && blk->where.count(p.second->data) == 0)
                blk->where[p.second->data] =
                    make_pair(1, blk->pack(blk->site, p.second->data, p.second->total_memory));
        g_blk = blk.get();
        return true;
    }
    void end_blocking(bool right) const {
        g_blk = nullptr;
        BlockRecorder &R = *blk;
        if (R.kr_am.empty()) {
            // nothing contracted here (every operator delayed): wait for the next one
            dumper->want_blocking = true;
            blk.reset();
            return;
        }
        vector<double> out(R.out_size, 0.0);
        size_t pos = 0;
        for (auto &o : R.out_list) {
            memcpy(out.data() + pos, o.first, sizeof(double) * o.second);
            pos += o.second;
        }
        Writer w(dumper->blk_dir);
        w.scalar("right", right);
        w.scalar("n_iadd", (double)R.ia_m.size());
        w.scalar("n_kron", (double)R.kr_am.size());
        w.scalar("tmp_size", (double)R.tmp_size);
        w.vec("ia_m", R.ia_m, "i4"), w.vec("ia_n", R.ia_n, "i4"), w.vec("ia_conj", R.ia_conj, "i4");
        w.vec("ia_dst", R.ia_dst, "u8"), w.vec("ia_src", R.ia_src, "u8");
        w.vec("ia_src_blob", R.ia_src_blob, "i4"), w.vec("ia_f", R.ia_f, "f8");
        w.vec("kr_am", R.kr_am, "i4"), w.vec("kr_an", R.kr_an, "i4"), w.vec("kr_ca", R.kr_ca, "i4");
        w.vec("kr_bm", R.kr_bm, "i4"), w.vec("kr_bn", R.kr_bn, "i4"), w.vec("kr_cb", R.kr_cb, "i4");
        w.vec("kr_cn", R.kr_cn, "i4"), w.vec("kr_ablob", R.kr_ablob, "i4");
        w.vec("kr_bblob", R.kr_bblob, "i4"), w.vec("kr_a", R.kr_a, "u8"), w.vec("kr_b", R.kr_b, "u8");
        w.vec("kr_c", R.kr_c, "u8"), w.vec("kr_f", R.kr_f, "f8");
        w.vec("env", R.env, "f8"), w.vec("site", R.site, "f8"), w.vec("out", out, "f8");
        w.man.flush();
        blk.reset();
    }
    // the fast expectation of one site (see NpdmRecorder): the reference's values,
    // its partials recorded by RecordingOpf, and the dot terms that combine them
    vector<pair<shared_ptr<OpExpr<S>>, double>>
    tensor_product_expectation(const vector<shared_ptr<OpExpr<S>>> &names,
                               const vector<shared_ptr<OpExpr<S>>> &exprs,
                               const shared_ptr<OperatorTensor<S, double>> &lopt,
                               const shared_ptr<OperatorTensor<S, double>> &ropt,
                               const shared_ptr<SparseMatrix<S, double>> &cmat,
                               const shared_ptr<SparseMatrix<S, double>> &vmat,
                               bool all_reduce) const override {
        NpdmRecorder *R = g_npdm;
        const bool rec = R != nullptr && R->calls++ == R->want;
        if (rec) {
            R->active = true;
            R->ket = cmat->data, R->nket = cmat->total_memory;
            R->bra = vmat->data, R->nbra = vmat->total_memory;
        }
        auto res = TF::tensor_product_expectation(names, exprs, lopt, ropt, cmat, vmat, all_reduce);
        if (!rec)
            return res;
        R->active = false;
        // dot terms, restating the last loops of tensor_product_expectation
        // (tensor_functions.hpp:1809-1872): expectation k = sum over its products
        // a x b of factor * dot(partial(conj, dq(b), opdq, a), b)
        vector<int32_t> t_k, t_part;
        vector<uint64_t> t_roff, t_rsize;
        vector<double> t_f, rblob, expect(names.size(), 0.0);
        map<const double *, size_t> roff;
        S ket_dq = cmat->info->delta_quantum, bra_dq = vmat->info->delta_quantum;
        for (size_t k = 0; k < exprs.size(); k++) {
            expect[k] = res[k].second;
            S opdq = dynamic_pointer_cast<OpElement<S, double>>(names[k])->q_label;
            if (opdq.combine(bra_dq, ket_dq) == S(S::invalid))
                continue;
            vector<shared_ptr<OpProduct<S, double>>> prods;
            if (exprs[k]->get_type() == OpTypes::Prod)
                prods.push_back(dynamic_pointer_cast<OpProduct<S, double>>(exprs[k]));
            else if (exprs[k]->get_type() == OpTypes::Sum)
                prods = dynamic_pointer_cast<OpSum<S, double>>(exprs[k])->strings;
            else if (exprs[k]->get_type() != OpTypes::Zero)
                throw runtime_error("npdm recorder: unexpected expression type");
            for (auto &op : prods) {
                auto rmat = ropt->ops.at(op->b);
                auto lmat = lopt->ops.at(op->a);
                auto it = R->part_key.find(make_tuple((int)op->conj, (uint64_t)rmat->info->delta_quantum.data,
                                                      (uint64_t)opdq.data, (const double *)lmat->data));
                if (it == R->part_key.end())
                    throw runtime_error("npdm recorder: a term without its partial");
                if (roff.count(rmat->data) == 0) {
                    roff[rmat->data] = rblob.size();
                    rblob.insert(rblob.end(), rmat->data, rmat->data + rmat->total_memory);
                }
                t_k.push_back((int32_t)k), t_part.push_back(it->second);
                t_roff.push_back(roff[rmat->data]), t_rsize.push_back(rmat->total_memory);
                t_f.push_back(op->factor);
            }
        }
        vector<double> ops(R->ket, R->ket + R->nket);
        if (R->bra != R->ket)
            ops.insert(ops.end(), R->bra, R->bra + R->nbra);
        vector<uint64_t> p_off, b_off;
        vector<int32_t> p_trans, p_nblk, b_rows, b_cols;
        for (auto &P : R->parts) {
            p_off.push_back(P.off), p_trans.push_back(P.trans), p_nblk.push_back((int32_t)P.rows.size());
            for (size_t q = 0; q < P.rows.size(); q++)
                b_rows.push_back(P.rows[q]), b_cols.push_back(P.cols[q]), b_off.push_back(P.off + P.boff[q]);
        }
        Writer w(R->out);
        w.scalar("n_pairs", (double)R->tb0.size()), w.scalar("n_partials", (double)R->parts.size());
        w.scalar("n_expect", (double)names.size()), w.scalar("n_terms", (double)t_k.size());
        w.scalar("psi_size", (double)R->lops.size()), w.scalar("ops_size", (double)ops.size());
        w.scalar("sigma_size", (double)R->sig), w.scalar("bra_is_ket", R->bra == R->ket);
        w.vec("tb0", R->tb0, "i4"), w.vec("m0", R->m0, "i4"), w.vec("n0", R->n0, "i4"), w.vec("k0", R->k0, "i4");
        w.vec("lda0", R->lda0, "i4"), w.vec("ldb0", R->ldb0, "i4"), w.vec("ta1", R->ta1, "i4");
        w.vec("m1", R->m1, "i4"), w.vec("n1", R->n1, "i4"), w.vec("k1", R->k1, "i4"), w.vec("lda1", R->lda1, "i4");
        w.vec("ldc1", R->ldc1, "i4"), w.vec("alpha0", R->al0, "f8"), w.vec("alpha1", R->al1, "f8");
        w.vec("a0", R->a0, "u8"), w.vec("b0", R->b0, "u8"), w.vec("a1", R->a1, "u8"), w.vec("c1", R->c1, "u8");
        w.vec("psi", R->lops, "f8"), w.vec("ops", ops, "f8"), w.vec("sigma", R->ref, "f8");
        w.vec("p_off", p_off, "u8"), w.vec("p_trans", p_trans, "i4"), w.vec("p_nblk", p_nblk, "i4");
        w.vec("b_off", b_off, "u8"), w.vec("b_rows", b_rows, "i4"), w.vec("b_cols", b_cols, "i4");
        w.vec("t_k", t_k, "i4"), w.vec("t_part", t_part, "i4"), w.vec("t_roff", t_roff, "u8");
        w.vec("t_rsize", t_rsize, "u8"), w.vec("t_f", t_f, "f8"), w.vec("rmats", rblob, "f8");
        w.vec("expect", expect, "f8");
        w.man.flush();
        return res;
    }
    void left_rotate(const shared_ptr<OperatorTensor<S, double>> &a,
                     const shared_ptr<SparseMatrix<S, double>> &bra,
                     const shared_ptr<SparseMatrix<S, double>> &ket,
                     shared_ptr<OperatorTensor<S, double>> &c) const override {
        TF::left_rotate(a, bra, ket, c);
        record(a->lmat, a, bra, ket, c, false);
    }
    void right_rotate(const shared_ptr<OperatorTensor<S, double>> &a,
                      const shared_ptr<SparseMatrix<S, double>> &bra,
                      const shared_ptr<SparseMatrix<S, double>> &ket,
                      shared_ptr<OperatorTensor<S, double>> &c) const override {
        TF::right_rotate(a, bra, ket, c);
        record(a->rmat, a, bra, ket, c, true);
    }
    void record(const shared_ptr<Symbolic<S>> &mat, const shared_ptr<OperatorTensor<S, double>> &a,
                const shared_ptr<SparseMatrix<S, double>> &bra,
                const shared_ptr<SparseMatrix<S, double>> &ket,
                const shared_ptr<OperatorTensor<S, double>> &c, bool trans) const {
        if (dumper == nullptr || !dumper->want_rotation)
            return;
        dumper->want_rotation = false;
        // packed blobs: input ops (psi role), rotated ops (sigma role), bra+ket (ops role)
        map<const double *, size_t> in_off, out_off;
        vector<double> in_blob, out_blob, mps_blob;
        auto pack = [](map<const double *, size_t> &off, vector<double> &blob,
                       const shared_ptr<SparseMatrix<S, double>> &m) {
            auto it = off.find(m->data);
            if (it != off.end())
                return it->second;
            size_t o = blob.size();
            off[m->data] = o;
            blob.insert(blob.end(), m->data, m->data + m->total_memory);
            return o;
        };
        const size_t bra_off = 0;
        mps_blob.insert(mps_blob.end(), bra->data, bra->data + bra->total_memory);
        const size_t ket_off = bra == ket ? 0 : mps_blob.size();
        if (bra != ket)
            mps_blob.insert(mps_blob.end(), ket->data, ket->data + ket->total_memory);
        vector<int32_t> tb0, m0, n0, k0, lda0, ldb0, ta1, m1, n1, k1, lda1, ldc1;
        vector<double> al0, al1;
        vector<uint64_t> a0, b0, a1, c1;
        for (size_t i = 0; i < mat->data.size(); i++) {
            if (mat->data[i]->get_type() == OpTypes::Zero)
                continue;
            auto pa = abs_value(mat->data[i]);
            auto A = a->ops.at(pa), C = c->ops.at(pa);
            const double scale = A->factor * bra->factor * ket->factor;
            if (abs(scale) < TINY)
                continue;
            const size_t ao = pack(in_off, in_blob, A), co = pack(out_off, out_blob, C);
            S cdq = C->info->delta_quantum;
            for (int ic = 0, ia = 0; ic < C->info->n; ia++, ic++) {
                while (A->info->quanta[ia] != C->info->quanta[ic])
                    ia++;
                S cq = C->info->quanta[ic].get_bra(cdq), cqp = C->info->quanta[ic].get_ket();
                int ibra = bra->info->find_state(cq), iket = ket->info->find_state(cqp);
                GMatrix<double> ma = (*A)[ia], mc = (*C)[ic], mb = (*bra)[ibra], mk = (*ket)[iket];
                const int cb = trans ? 0 : 1, ck = trans ? 1 : 0;  // conj bits (!trans|2)&1, trans&1
                tb0.push_back(ck), m0.push_back(ma.m), k0.push_back(ma.n), lda0.push_back(ma.n);
                n0.push_back(ck ? mk.m : mk.n), ldb0.push_back(mk.n);
                ta1.push_back(cb), m1.push_back(mc.m), k1.push_back(ma.m), lda1.push_back(mb.n);
                n1.push_back(mc.n), ldc1.push_back(mc.n);
                al0.push_back(1.0), al1.push_back(scale);
                a0.push_back(ao + (ma.data - A->data)), b0.push_back(ket_off + (mk.data - ket->data));
                a1.push_back(bra_off + (mb.data - bra->data)), c1.push_back(co + (mc.data - C->data));
            }
        }
        Writer w(dumper->rot_dir);
        w.scalar("n_pairs", (double)tb0.size());
        w.scalar("psi_size", (double)in_blob.size());
        w.scalar("sigma_size", (double)out_blob.size());
        w.scalar("ops_size", (double)mps_blob.size());
        w.scalar("trans", trans);
        w.vec("tb0", tb0, "i4"), w.vec("m0", m0, "i4"), w.vec("n0", n0, "i4"), w.vec("k0", k0, "i4");
        w.vec("lda0", lda0, "i4"), w.vec("ldb0", ldb0, "i4"), w.vec("ta1", ta1, "i4");
        w.vec("m1", m1, "i4"), w.vec("n1", n1, "i4"), w.vec("k1", k1, "i4"), w.vec("lda1", lda1, "i4");
        w.vec("ldc1", ldc1, "i4"), w.vec("alpha0", al0, "f8"), w.vec("alpha1", al1, "f8");
        w.vec("a0", a0, "u8"), w.vec("b0", b0, "u8"), w.vec("a1", a1, "u8"), w.vec("c1", c1, "u8");
        w.vec("psi", in_blob, "f8"), w.vec("ops", mps_blob, "f8"), w.vec("sigma", out_blob, "f8");
        w.man.flush();
    }
};

template <typename S>
shared_ptr<MPO<S, double>> qc_mpo(const shared_ptr<HamiltonianQC<S, double>> &hamil) {
    shared_ptr<MPO<S, double>> mpo = make_shared<MPOQC<S, double>>(hamil, QCTypes::Conventional, "HQC");
    return make_shared<SimplifiedMPO<S, double>>(mpo, make_shared<RuleQC<S, double>>(), true, true,
                                                 OpNamesSet({OpNames::R, OpNames::RD}));
}

// Per perturbed Hamiltonian, the H_eff at one site of the final MPS built with
// it (a copy of the final MPS with its canonical centre moved to that site,
// dumped by a one-site sweep before its Davidson changes anything); then the
// reference's 1-/2-PDM of the final MPS (Expect with PDM1MPOQC / PDM2MPOQC,
// the pattern of unit_test/test_npdm_n2_sto3g.cpp).
template <typename S>
void fixed_mps_outputs(const Opts &o, const shared_ptr<HamiltonianQC<S, double>> &hamil,
                       const shared_ptr<MPS<S, double>> &mps, int n) {
    typedef double FL;
    mps->save_data();
    shared_ptr<Threading> saved_threading = threading_();
    if (o.perturb_threads > 0) {
        threading_() = make_shared<Threading>(ThreadingTypes::OperatorBatchedGEMM | ThreadingTypes::Global,
                                              o.perturb_threads, o.perturb_threads, 1);
        threading_()->seq_type = SeqTypes::Tasked;
    }
    for (size_t k = 0; k < o.perturb.size(); k++) {
        auto fd = make_shared<FCIDUMP<FL>>();
        fd->read(o.perturb[k]);
        vector<uint8_t> orbsym(n, 0);
        auto ham2 = make_shared<HamiltonianQC<S, FL>>(hamil->vacuum, n, orbsym, fd);
        shared_ptr<MPO<S, FL>> mpo2 = qc_mpo<S>(ham2);
        auto xmps = mps->deep_copy("PT" + to_string(k));
        // walk the centre from the left end to the requested site with a
        // sweep whose Davidson stops at its initial guess (the current
        // two-site wavefunction): each split keeps every state (the MPS is
        // already truncated to M), so the state stays the converged one
        const int target = o.perturb_site >= 0 ? o.perturb_site : n / 2 - 1;
        if (xmps->center != 0)
            throw runtime_error("fixed-MPS perturbation expects the final MPS centre at site 0");
        auto dumper = make_shared<Dumper<S>>();
        dumper->o = o;
        dumper->o.dump_sweep = 0;
        dumper->o.dump_site = target;
        dumper->o.dump_dm = false;
        dumper->o.out = o.out + "/perturb" + to_string(k);
        auto me2 = make_shared<MovingEnvironment<S, FL, FL>>(mpo2, xmps, xmps, "PT" + to_string(k));
        me2->init_environments(false);
        me2->delayed_contraction = OpNamesSet::normal_ops();
        me2->cached_contraction = true;
        vector<ubond_t> bdims = {(ubond_t)o.M};
        auto dmrg2 = make_shared<DMRG<S, FL, FL>>(me2, bdims, vector<FL>{0.0});
        dmrg2->davidson_conv_thrds = vector<FL>{1e10};
        dmrg2->noise_type = NoiseTypes::DensityMatrix;
        dmrg2->iprint = 0;
        dmrg2->sweep_start_site = 0;
        dmrg2->sweep_end_site = target + 2;
        dumper->d = dmrg2.get();
        callback_() = dumper;
        dmrg2->solve(1, true, 0.0);
        callback_() = make_shared<CallbackKernel>();
        mpo2->deallocate();
        me2->remove_partition_files();
    }
    threading_() = saved_threading;
    if (o.pdm) {
        Writer w(o.out + "/pdm");
        for (int k = 1; k <= 2; k++) {
            shared_ptr<MPO<S, FL>> pmpo;
            if (k == 1)
                pmpo = make_shared<PDM1MPOQC<S, FL>>(hamil);
            else
                pmpo = make_shared<PDM2MPOQC<S, FL>>(hamil);
            pmpo = make_shared<SimplifiedMPO<S, FL>>(pmpo, make_shared<RuleQC<S, FL>>(), true, true,
                                                    OpNamesSet({OpNames::R, OpNames::RD}));
            NpdmRecorder npdm;
            if (k == o.npdm_order && o.npdm_call >= 0) {
                // the fast expectations of that PDM sweep go through the recording
                // tensor functions; the chosen one is written (NpdmRecorder)
                auto ropf = make_shared<RecordingOpf<S>>(pmpo->tf->opf->cg);
                ropf->seq = pmpo->tf->opf->seq;
                pmpo->tf = make_shared<RecordingTF<S>>(ropf, nullptr);
                npdm.want = o.npdm_call, npdm.out = o.out + "/npdm_product";
                g_npdm = &npdm;
            }
            auto pme = make_shared<MovingEnvironment<S, FL, FL>>(pmpo, mps, mps, k == 1 ? "1PDM" : "2PDM");
            pme->init_environments(false);
            auto ex = make_shared<Expect<S, FL, FL>>(pme, (ubond_t)o.M, (ubond_t)o.M);
            ex->solve(true, mps->center == 0);
            g_npdm = nullptr;
            if (k == 1) {
                GMatrix<FL> dm = ex->get_1pdm_spatial();
                vector<double> v(dm.data, dm.data + (size_t)n * n);
                w.vec("dm1", v, "f8");
                dm.deallocate();
            } else {
                shared_ptr<GTensor<FL>> dm2 = ex->get_2pdm_spatial();
                w.vec("dm2", *dm2->data, "f8");
            }
            pmpo->deallocate();
            pme->remove_partition_files();
        }
        w.scalar("n", n);
        w.man.flush();
    }
}

template <typename S> int run(const Opts &o) {
    typedef double FL;
    Random::rand_seed(o.seed);
    string scratch = o.out + "/_scratch";
    mkdirs(scratch);
    frame_<FL>() = make_shared<DataFrame<FL>>((size_t)1 << 26, (size_t)1 << 32, scratch);
    frame_<FL>()->use_main_stack = false;
    frame_<FL>()->minimal_disk_usage = true;
    threading_() = make_shared<Threading>(
        ThreadingTypes::OperatorBatchedGEMM | ThreadingTypes::Global, o.nthreads, o.nthreads, 1);
    threading_()->seq_type = SeqTypes::Tasked;
    shared_ptr<FCIDUMP<FL>> fcidump;
    if (o.ham == "hubbard")
        fcidump = make_shared<HubbardFCIDUMP>(o.L, o.t, o.U);
    else {
        fcidump = make_shared<FCIDUMP<FL>>();
        fcidump->read(o.ham);
    }
    const int n = fcidump->n_sites();
    vector<uint8_t> orbsym(n, 0); // no point-group symmetry in these Hamiltonians
    S vacuum(0);
    S target(fcidump->n_elec(), fcidump->twos(), 0);
    auto hamil = make_shared<HamiltonianQC<S, FL>>(vacuum, n, orbsym, fcidump);
    shared_ptr<MPO<S, FL>> mpo = make_shared<MPOQC<S, FL>>(hamil, QCTypes::Conventional, "HQC");
    mpo = make_shared<SimplifiedMPO<S, FL>>(mpo, make_shared<RuleQC<S, FL>>(), true, true,
                                            OpNamesSet({OpNames::R, OpNames::RD}));
    auto mps_info = make_shared<MPSInfo<S>>(n, vacuum, target, hamil->basis);
    mps_info->set_bond_dimension(o.M);
    auto mps = make_shared<MPS<S, FL>>(n, 0, 2);
    mps->initialize(mps_info);
    mps->random_canonicalize();
    mps->save_mutable();
    mps->deallocate();
    mps_info->save_mutable();
    mps_info->deallocate_mutable();
    auto dumper = make_shared<Dumper<S>>();
    dumper->o = o;
    {
        auto ropf = make_shared<RecordingOpf<S>>(mpo->tf->opf->cg);
        ropf->seq = mpo->tf->opf->seq;
        mpo->tf = make_shared<RecordingTF<S>>(ropf, dumper.get());
    }
    auto me = make_shared<MovingEnvironment<S, FL, FL>>(mpo, mps, mps, "DMRG");
    me->init_environments(false);
    me->delayed_contraction = OpNamesSet::normal_ops();
    me->cached_contraction = true;
    vector<ubond_t> bdims = {(ubond_t)o.M};
    auto dmrg = make_shared<DMRG<S, FL, FL>>(me, bdims, o.noises);
    dmrg->davidson_conv_thrds = o.dav_thrds;
    dmrg->noise_type = NoiseTypes::DensityMatrix;
    dmrg->iprint = 2;
    dumper->d = dmrg.get();
    callback_() = dumper;
    Timer t;
    t.get_time();
    double e = dmrg->solve(o.nsweeps, true, o.tol);
    double tt = t.get_time();
    callback_() = make_shared<CallbackKernel>();
    Writer w(o.out + "/result");
    w.scalar("energy", e);
    w.scalar("time", tt);
    w.scalar("n_sites", n);
    vector<double> es, dws;
    for (auto &x : dmrg->energies)
        es.push_back(x.back());
    for (auto &x : dmrg->discarded_weights)
        dws.push_back(x);
    w.vec("sweep_energies", es, "f8");
    w.vec("discarded_weights", dws, "f8");
    cout << setprecision(12) << "FINAL E = " << e << " T = " << tt << endl;
    if (o.pdm || !o.perturb.empty())
        fixed_mps_outputs<S>(o, hamil, mps, n);
    mps_info->deallocate();
    mpo->deallocate();
    me->remove_partition_files();
    return 0;
}

static vector<double> parse_list(const string &s) {
    vector<double> r;
    stringstream ss(s);
    string x;
    while (getline(ss, x, ','))
        r.push_back(atof(x.c_str()));
    return r;
}

} // namespace harness

int main(int argc, char **argv) {
    harness::Opts o;
    for (int i = 1; i + 1 < argc; i += 2) {
        string k = argv[i], v = argv[i + 1];
        if (k == "--ham") o.ham = v;
        else if (k == "--L") o.L = atoi(v.c_str());
        else if (k == "--t") o.t = atof(v.c_str());
        else if (k == "--U") o.U = atof(v.c_str());
        else if (k == "--sym") o.sym = v;
        else if (k == "--M") o.M = atoi(v.c_str());
        else if (k == "--sweeps") o.nsweeps = atoi(v.c_str());
        else if (k == "--threads") o.nthreads = atoi(v.c_str());
        else if (k == "--seed") o.seed = atoi(v.c_str());
        else if (k == "--noises") o.noises = harness::parse_list(v);
        else if (k == "--dav") o.dav_thrds = harness::parse_list(v);
        else if (k == "--tol") o.tol = atof(v.c_str());
        else if (k == "--out") o.out = v;
        else if (k == "--dump-sweep") o.dump_sweep = atoi(v.c_str());
        else if (k == "--dump-site") o.dump_site = atoi(v.c_str());
        else if (k == "--with-data") o.with_data = atoi(v.c_str()) != 0;
        else if (k == "--pdm") o.pdm = atoi(v.c_str()) != 0;
        else if (k == "--effprob") o.effprob = atoi(v.c_str()) != 0;
        else if (k == "--noise-product") o.noise = atoi(v.c_str());
        else if (k == "--perturb-site") o.perturb_site = atoi(v.c_str());
        else if (k == "--perturb-threads") o.perturb_threads = atoi(v.c_str());
        else if (k == "--npdm-product") o.npdm_call = atoi(v.c_str());
        else if (k == "--npdm-order") o.npdm_order = atoi(v.c_str());
        else if (k == "--perturb") {
            stringstream ss(v);
            string x;
            while (getline(ss, x, ','))
                o.perturb.push_back(x);
        }
        else {
            cerr << "unknown option " << k << endl;
            return 2;
        }
    }
    if (o.sym == "su2")
        return harness::run<SU2>(o);
    else if (o.sym == "sz")
        return harness::run<SZ>(o);
    cerr << "unknown symmetry " << o.sym << endl;
    return 2;
}
