// dmrg_sweep.cpp -- runs block2's own two-site DMRG (DMRG::solve, unchanged)
// on one Hamiltonian, on the host cores or with the GB300 drop-in installed.
//
// The set-up is block2's documented C++ pattern for a quantum-chemistry DMRG
// (unit_test/test_dmrg_n2_sto3g.cpp:47-120): FCIDUMP (or the Hubbard chain,
// src/core/hubbard.hpp:31) -> HamiltonianQC -> MPOQC(Conventional) +
// SimplifiedMPO(RuleQC) -> MPSInfo / MPS::random_canonicalize ->
// MovingEnvironment (delayed + cached contraction) -> DMRG::solve, with
// Threading OperatorBatchedGEMM|Global and SeqTypes::Tasked (block2's driver
// defaults, pyblock2/driver/core.py:696-705).
//
// A run has up to two stages, each a DMRG::solve:
//   warm-up  (--warm-sweeps W, optional) on --warm-device from the random MPS;
//   arms     (--arms, default "cpu") one solve of --sweeps sweeps per arm, each
//            on its own copy (MPS::deep_copy) of the MPS the warm-up left, with
//            its own MovingEnvironment; so every arm starts from the same state
//            with the same schedule, and arms can be compared sweep by sweep.
// An arm is "cpu" (block2's own CPU path) or "gpu:FORM" (FORM = fp64, tf32x3,
// fp32), optionally with "/K" to run K sweeps instead of --sweeps, "@E" to
// stop a single forward sweep at site E (a partial sweep) and "%T" to solve
// every Davidson problem of the arm to tolerance T instead of --dav; a GPU arm has
// b2g_block2::GpuTensorFunctions installed as mpo->tf and
// b2g_block2::GpuDMRG as the sweep driver, so every Davidson solve runs on the
// device.  Built with -DB2G_REFERENCE_ONLY the program has no GPU code at all
// and accepts only cpu arms.
//
// Output (--json): per stage and arm, the sweep energies, discarded weights,
// per-sweep wall times and the reference's per-phase timers, and the block
// structure of every site tensor of the final MPS (quanta and block shapes).
#include "block2_core.hpp"
#include "block2_dmrg.hpp"
#ifndef B2G_REFERENCE_ONLY
#include "b2g_block2.hpp"
#endif
#include <sys/stat.h>

using namespace block2;

namespace sweep_driver {

struct Schedule {
    vector<double> bond_dims = {250};
    vector<double> noises = {0.0};
    vector<double> dav_thrds = {1e-10};
    int nsweeps = 4;
};

struct Opts {
    string ham = "hubbard";
    int L = 16;
    double t = 1.0, U = 4.0;
    string sym = "su2";
    int nthreads = 4, iprint = 2, nroots = 1;  // nroots > 1: state-averaged MultiMPS
    unsigned seed = 1234;  // block2 seeds from the clock when given 0
    Schedule sched, warm = Schedule{{250}, {0.0}, {1e-10}, 0};  // no warm-up unless asked
    string warm_device = "cpu";
    vector<string> arms = {"cpu"};
    double tol = 0.0;
    string json, scratch = "";
    double stack_gb = 4.0;  // block2's DataFrame stack (its second frame holds 30 % of it)
    // noise: "dm" (NoiseTypes::DensityMatrix), "perturbative" (ReducedPerturbative),
    // "perturbative-full" (Perturbative), "perturbative-lowmem" (ReducedPerturbativeLowMem) or
    // "perturbative-collected" (ReducedPerturbativeCollected, pyblock2's driver default);
    // noise_on_device: GPU arms run the perturbative-noise product on the device
    string noise_type = "dm";
    int noise_on_device = 1;
    // after each arm: block2's 1-PDM (Expect with PDM1MPOQC) of the arm's final MPS,
    // on the arm's device (GPU arms: the fast expectation's partials on the GPU);
    // 2: GPU arms also compute it with block2's own tensor functions
    int pdm = 0;
    int pdm_on_gpu = 0;  // 1: the PDM goes through the drop-in after CPU arms too
    int pdm_order = 1;   // 1: the 1-PDM (PDM1MPOQC); 2: the 2-PDM (PDM2MPOQC)
    int start_site = 0, end_site = -1;  // restricts every arm's sweeps (timing samples)
    // GPU stages: dump the H_eff of one site of one sweep of arm dump_arm
    // (-1: of the warm-up)
    string dump_dir;
    int dump_arm = 0, dump_sweep = -1, dump_site = -1;
};

static void mkdirs(const string &p) {
    string cur;
    for (size_t i = 0; i < p.size(); i++) {
        cur.push_back(p[i]);
        if (p[i] == '/' || i + 1 == p.size())
            mkdir(cur.c_str(), 0755);
    }
}

struct SweepPhase {
    double wall, teff, teig, tprt, tblk, tmve, tdm, tsplt, trot, tctr, tmid, tint, tdctr, tdiag, tinfo;
    // GPU arms: time inside the device Davidson solves, the pair translation
    // and the plan build + operator upload during the sweep
    double gdav = 0, gtranslate = 0, gplan = 0, h2d = 0, d2h = 0;
    double nflop = 0;  // block2's multiply-add counter of the sweep (sweep_cumulative_nflop)
};

// Times each sweep and reads the reference's own per-phase timers when it
// ends (DMRG::sweep raises "DMRG::sweep.start" before its first site and
// "DMRG::sweep.end" after its last, src/dmrg/sweep_algorithm.hpp:2593, 2662).
template <typename S> struct PhaseRecorder : CallbackKernel {
    DMRG<S, double, double> *d = nullptr;
    mutable vector<SweepPhase> phases;
    mutable Timer t;
#ifndef B2G_REFERENCE_ONLY
    b2g_block2::Runtime *rt = nullptr;
    mutable double g0[5] = {0, 0, 0, 0, 0};
#endif
    void compute(const string &name, int iprint) const override {
        if (d == nullptr)
            return;
        if (name == "DMRG::sweep.start") {
#ifndef B2G_REFERENCE_ONLY
            if (rt != nullptr)
                g0[0] = rt->t_davidson, g0[1] = rt->t_plan, g0[2] = rt->t_upload, g0[3] = rt->h2d_bytes,
                g0[4] = rt->d2h_bytes;
#endif
            t.get_time();
        }
        if (name != "DMRG::sweep.end")
            return;
        auto &me = *d->me;
        SweepPhase p{t.get_time(), d->teff, d->teig, d->tprt, d->tblk, d->tmve, d->tdm,
                     d->tsplt, me.trot, me.tctr, me.tmid, me.tint, me.tdctr, me.tdiag, me.tinfo};
#ifndef B2G_REFERENCE_ONLY
        if (rt != nullptr)
            p.gdav = rt->t_davidson - g0[0], p.gtranslate = rt->t_plan - g0[1], p.gplan = rt->t_upload - g0[2],
            p.h2d = rt->h2d_bytes - g0[3], p.d2h = rt->d2h_bytes - g0[4];
#endif
        p.nflop = (double)d->sweep_cumulative_nflop;
        phases.push_back(p);
    }
};

template <typename T> static void json_list(ostream &os, const vector<T> &v) {
    os << "[";
    for (size_t i = 0; i < v.size(); i++)
        os << (i ? ", " : "") << v[i];
    os << "]";
}

template <typename S> struct Problem {
    typedef double FL;
    shared_ptr<HamiltonianQC<S, FL>> hamil;
    shared_ptr<MPO<S, FL>> mpo;
    shared_ptr<TensorFunctions<S, FL>> cpu_tf;  // block2's own tensor functions
    int n = 0;
#ifndef B2G_REFERENCE_ONLY
    shared_ptr<b2g_block2::Runtime> rt;
#endif
};

// One DMRG::solve on `mps` with the given device; writes the stage's results.
template <typename S>
void solve_stage(Problem<S> &pb, const shared_ptr<MPS<S, double>> &mps, const string &device,
                 const Schedule &sc, const Opts &o, bool forward, const string &tag, ostream &js) {
    typedef double FL;
    string dev = device, form = "fp64";
    if (dev.find(':') != string::npos)
        form = dev.substr(dev.find(':') + 1), dev = dev.substr(0, dev.find(':'));
    // gpu: GpuDMRG (device Davidson); gpuop: the drop-in's tensor functions under
    // block2's own DMRG and host Davidson (every product through the C ABI)
    const bool gpu = dev == "gpu" || dev == "gpuop", host_davidson = dev == "gpuop";
    if (!gpu && dev != "cpu")
        throw runtime_error("unknown device " + device);
    pb.mpo->tf = pb.cpu_tf;
#ifndef B2G_REFERENCE_ONLY
    if (gpu) {
        const int f = form == "fp64" ? B2G_FP64 : form == "tf32x3" ? B2G_TF32X3 : form == "fp32" ? B2G_FP32 : -1;
        if (f < 0)
            throw runtime_error("unknown GPU form " + form);
        if (pb.rt == nullptr)
            pb.rt = make_shared<b2g_block2::Runtime>(0, f);
        pb.rt->form = f;
        pb.rt->n_heff = pb.rt->n_apply_fp64 = pb.rt->n_apply_reduced = pb.rt->n_noise = 0;
        pb.rt->noise_on_device = o.noise_on_device != 0;
        pb.rt->t_plan = pb.rt->t_upload = pb.rt->t_davidson = 0;
        b2g_block2::install<S>(pb.mpo, pb.rt);
    }
#else
    if (gpu)
        throw runtime_error("this build is block2's CPU path only (B2G_REFERENCE_ONLY)");
#endif
    vector<ubond_t> bdims;
    for (double b : sc.bond_dims)
        bdims.push_back((ubond_t)b);
    auto me = make_shared<MovingEnvironment<S, FL, FL>>(pb.mpo, mps, mps, tag);
    me->init_environments(false);
    me->delayed_contraction = OpNamesSet::normal_ops();
    me->cached_contraction = true;
    shared_ptr<DMRG<S, FL, FL>> dmrg;
#ifndef B2G_REFERENCE_ONLY
    if (gpu && !host_davidson) {
        auto gd = make_shared<b2g_block2::GpuDMRG<S>>(me, bdims, sc.noises, pb.rt);
        if (!o.dump_dir.empty() && tag == (o.dump_arm < 0 ? string("WARM") : "ARM" + to_string(o.dump_arm))) {
            mkdirs(o.dump_dir);
            gd->dump_dir = o.dump_dir, gd->dump_sweep = o.dump_sweep;
            gd->dump_site = o.dump_site >= 0 ? o.dump_site : pb.n / 2 - 1;
        }
        dmrg = gd;
    } else
#endif
        dmrg = make_shared<DMRG<S, FL, FL>>(me, bdims, sc.noises);
    dmrg->davidson_conv_thrds = sc.dav_thrds;
    if (o.noise_type == "dm")
        dmrg->noise_type = NoiseTypes::DensityMatrix;
    else if (o.noise_type == "perturbative")
        dmrg->noise_type = NoiseTypes::ReducedPerturbative;
    else if (o.noise_type == "perturbative-full")
        dmrg->noise_type = NoiseTypes::Perturbative;
    else if (o.noise_type == "perturbative-lowmem")
        dmrg->noise_type = NoiseTypes::ReducedPerturbativeLowMem;
    else if (o.noise_type == "perturbative-collected")
        dmrg->noise_type = NoiseTypes::ReducedPerturbativeCollected;
    else
        throw runtime_error("unknown noise type " + o.noise_type);
    dmrg->iprint = (uint8_t)o.iprint;
    dmrg->sweep_start_site = o.start_site;
    if (o.end_site > 0)
        dmrg->sweep_end_site = o.end_site;
    auto rec = make_shared<PhaseRecorder<S>>();
    rec->d = dmrg.get();
#ifndef B2G_REFERENCE_ONLY
    if (gpu)
        rec->rt = pb.rt.get();
#endif
    callback_() = rec;
    cout << "== stage " << tag << ": " << device << ", " << sc.nsweeps << " sweeps" << endl;
    uint64_t launches0 = 0;
#ifndef B2G_REFERENCE_ONLY
    if (gpu)
        b2g_launch_count(&launches0);
#endif
    Timer t;
    t.get_time();
    const double e = (double)dmrg->solve(sc.nsweeps, forward, o.tol);
    const double tt = t.get_time();
    callback_() = make_shared<CallbackKernel>();
    cout << setprecision(12) << "FINAL E (" << tag << ") = " << e << " T = " << tt << endl;
    js << "{\"tag\": \"" << tag << "\", \"device\": \"" << dev << "\", \"form\": \"" << (gpu ? form : "fp64")
       << "\", \"energy\": " << e << ", \"time\": " << tt;
    vector<double> es, dws, walls;
    for (auto &x : dmrg->energies)
        es.push_back((double)x.back());
    for (auto &x : dmrg->discarded_weights)
        dws.push_back((double)x);
    for (auto &p : rec->phases)
        walls.push_back(p.wall);
    js << ", \"sweep_energies\": ";
    json_list(js, es);
    js << ", \"sweep_energies_roots\": [";
    for (size_t q = 0; q < dmrg->energies.size(); q++) {
        vector<double> er(dmrg->energies[q].begin(), dmrg->energies[q].end());
        js << (q ? ", " : "");
        json_list(js, er);
    }
    js << "]";
    js << ", \"discarded_weights\": ";
    json_list(js, dws);
    js << ", \"sweep_time\": ";
    json_list(js, walls);
    js << ", \"phases\": [";
    for (size_t i = 0; i < rec->phases.size(); i++) {
        auto &p = rec->phases[i];
        js << (i ? ", " : "") << "{\"teff\": " << p.teff << ", \"teig\": " << p.teig << ", \"tprt\": " << p.tprt
           << ", \"tblk\": " << p.tblk << ", \"tmve\": " << p.tmve << ", \"tdm\": " << p.tdm
           << ", \"tsplt\": " << p.tsplt << ", \"trot\": " << p.trot << ", \"tctr\": " << p.tctr
           << ", \"tmid\": " << p.tmid << ", \"tint\": " << p.tint << ", \"tdctr\": " << p.tdctr
           << ", \"tdiag\": " << p.tdiag << ", \"tinfo\": " << p.tinfo << ", \"gpu_davidson\": " << p.gdav
           << ", \"gpu_translate\": " << p.gtranslate << ", \"gpu_plan_upload\": " << p.gplan
           << ", \"mnk\": " << p.nflop << ", \"h2d_bytes\": " << p.h2d << ", \"d2h_bytes\": " << p.d2h << "}";
    }
    js << "]";
    // block structure of the final MPS: per site tensor, each block's packed
    // quantum label and shape
    js << ", \"mps_blocks\": [";
    for (int i = 0; i < pb.n; i++) {
        if (mps->tensors[i] == nullptr) {
            js << (i ? ", " : "") << "null";
            continue;
        }
        mps->load_tensor(i);
        auto info = mps->tensors[i]->info;
        js << (i ? ", " : "") << "{\"form\": \"" << mps->canonical_form[i] << "\", \"q\": [";
        for (int b = 0; b < info->n; b++)
            js << (b ? ", " : "") << "\"" << info->quanta[b].data << "\"";
        js << "], \"rows\": [";
        for (int b = 0; b < info->n; b++)
            js << (b ? ", " : "") << info->n_states_bra[b];
        js << "], \"cols\": [";
        for (int b = 0; b < info->n; b++)
            js << (b ? ", " : "") << info->n_states_ket[b];
        js << "]}";
        mps->unload_tensor(i);
    }
    js << "]";
#ifndef B2G_REFERENCE_ONLY
    if (gpu)
        js << ", \"gpu\": {\"heff_plans\": " << pb.rt->n_heff << ", \"noise_products\": " << pb.rt->n_noise
           << ", \"apply_fp64\": " << pb.rt->n_apply_fp64
           << ", \"apply_reduced\": " << pb.rt->n_apply_reduced << ", \"t_translate\": " << pb.rt->t_plan
           << ", \"t_plan_upload\": " << pb.rt->t_upload << ", \"kernel_launches\": " << [&] {
                  uint64_t n1 = 0;
                  b2g_launch_count(&n1);
                  return n1 - launches0;
              }() << "}";
#endif
    if (o.pdm) {
        // the 1-PDM of this arm's final MPS (as block2's Expect computes it), on the
        // arm's device; --pdm 2 on a GPU arm also computes it with block2's own
        // tensor functions on the same MPS ("pdm1_host")
        mps->save_data();
        auto one_pdm = [&](bool on_gpu, const string &label, double &secs) {
            shared_ptr<MPO<S, FL>> pmpo;
            if (o.pdm_order == 2)
                pmpo = make_shared<PDM2MPOQC<S, FL>>(pb.hamil);
            else
                pmpo = make_shared<PDM1MPOQC<S, FL>>(pb.hamil);
            pmpo = make_shared<SimplifiedMPO<S, FL>>(pmpo, make_shared<RuleQC<S, FL>>(), true, true,
                                                    OpNamesSet({OpNames::R, OpNames::RD}));
#ifndef B2G_REFERENCE_ONLY
            if (on_gpu)
                b2g_block2::install<S>(pmpo, pb.rt);
#else
            (void)on_gpu;
#endif
            auto pme = make_shared<MovingEnvironment<S, FL, FL>>(pmpo, mps, mps, tag + label);
            pme->init_environments(false);
            const ubond_t bd = (ubond_t)sc.bond_dims.back();
            auto ex = make_shared<Expect<S, FL, FL>>(pme, bd, bd);
            ex->iprint = 0;
            Timer tp;
            tp.get_time();
            ex->solve(true, mps->center == 0);
            secs = tp.get_time();
            vector<double> v;
            if (o.pdm_order == 2) {
                shared_ptr<GTensor<FL>> dm2 = ex->get_2pdm_spatial();
                v.assign(dm2->data->begin(), dm2->data->end());
            } else {
                GMatrix<FL> dm = ex->get_1pdm_spatial();
                v.assign(dm.data, dm.data + (size_t)dm.m * dm.n);
                dm.deallocate();
            }
            pme->remove_partition_files();
            pmpo->deallocate();
            return v;
        };
        bool pdm_gpu = gpu;
#ifndef B2G_REFERENCE_ONLY
        if (o.pdm_on_gpu && !pb.rt)
            pb.rt = make_shared<b2g_block2::Runtime>(0, B2G_FP64);
        pdm_gpu = gpu || o.pdm_on_gpu;
        const long long nexp0 = pdm_gpu ? pb.rt->n_expect : 0;
#else
        if (o.pdm_on_gpu)
            throw runtime_error("this build is block2's CPU path only (B2G_REFERENCE_ONLY)");
#endif
        double tpdm = 0;
        const string key = o.pdm_order == 2 ? "pdm2" : "pdm1";  // JSON keys: pdm1* or pdm2*
        js << ", \"" << key << "\": ";
        json_list(js, one_pdm(pdm_gpu, "PDM", tpdm));
        js << ", \"" << key << "_time\": " << tpdm;
#ifndef B2G_REFERENCE_ONLY
        if (pdm_gpu) {
            js << ", \"" << key << "_device_products\": " << pb.rt->n_expect - nexp0;
            if (o.pdm == 2) {
                js << ", \"" << key << "_host\": ";
                json_list(js, one_pdm(false, "PDMH", tpdm));
                js << ", \"" << key << "_host_time\": " << tpdm;
            }
        }
#endif
    }
    js << "}";
    pb.mpo->tf = pb.cpu_tf;
    me->remove_partition_files();
}

template <typename S> int run(const Opts &o) {
    typedef double FL;
    Random::rand_seed(o.seed);
    const string scratch = o.scratch.empty() ? string("./nodex_b2g_sweep") : o.scratch;
    mkdirs(scratch);
    frame_<FL>() = make_shared<DataFrame<FL>>((size_t)1 << 26, (size_t)(o.stack_gb * (double)(1ull << 30)), scratch);
    frame_<FL>()->use_main_stack = false;
    frame_<FL>()->minimal_disk_usage = true;
    threading_() = make_shared<Threading>(ThreadingTypes::OperatorBatchedGEMM | ThreadingTypes::Global,
                                          o.nthreads, o.nthreads, 1);
    threading_()->seq_type = SeqTypes::Tasked;
    shared_ptr<FCIDUMP<FL>> fcidump;
    if (o.ham == "hubbard")
        fcidump = make_shared<HubbardFCIDUMP>(o.L, o.t, o.U);
    else {
        fcidump = make_shared<FCIDUMP<FL>>();
        fcidump->read(o.ham);
    }
    Problem<S> pb;
    pb.n = fcidump->n_sites();
    vector<uint8_t> orbsym(pb.n, 0);
    S vacuum(0);
    S target(fcidump->n_elec(), fcidump->twos(), 0);
    pb.hamil = make_shared<HamiltonianQC<S, FL>>(vacuum, pb.n, orbsym, fcidump);
    pb.mpo = make_shared<MPOQC<S, FL>>(pb.hamil, QCTypes::Conventional, "HQC");
    pb.mpo = make_shared<SimplifiedMPO<S, FL>>(pb.mpo, make_shared<RuleQC<S, FL>>(), true, true,
                                               OpNamesSet({OpNames::R, OpNames::RD}));
    pb.cpu_tf = pb.mpo->tf;
    const Schedule &first = o.warm.nsweeps > 0 ? o.warm : o.sched;
    shared_ptr<MPSInfo<S>> mps_info;
    shared_ptr<MPS<S, FL>> mps;
    if (o.nroots > 1) {
        // state-averaged roots of one target (block2's MultiMPS, equal weights)
        mps_info = make_shared<MultiMPSInfo<S>>(pb.n, vacuum, vector<S>{target}, pb.hamil->basis);
        mps = make_shared<MultiMPS<S, FL>>(pb.n, 0, 2, o.nroots);
    } else {
        mps_info = make_shared<MPSInfo<S>>(pb.n, vacuum, target, pb.hamil->basis);
        mps = make_shared<MPS<S, FL>>(pb.n, 0, 2);
    }
    mps_info->set_bond_dimension((ubond_t)first.bond_dims[0]);
    mps->initialize(mps_info);
    mps->random_canonicalize();
    mps->save_mutable();
    mps->deallocate();
    mps_info->save_mutable();
    mps_info->deallocate_mutable();
    stringstream js;
    js << setprecision(17);
    js << "{\"n_sites\": " << pb.n << ", \"threads\": " << o.nthreads << ", \"seed\": " << o.seed
       << ", \"const_e\": " << (double)pb.mpo->const_e;
    if (o.warm.nsweeps > 0) {
        if (o.warm.nsweeps % 2 != 0)
            throw runtime_error("--warm-sweeps must be even (the arms start forward from site 0)");
        js << ", \"warm\": ";
        solve_stage<S>(pb, mps, o.warm_device, o.warm, o, true, "WARM", js);
    }
    js << ", \"arms\": [";
    const bool copies = o.arms.size() > 1 || o.warm.nsweeps > 0;
    if (copies)
        mps->save_data();
    for (size_t a = 0; a < o.arms.size(); a++) {
        auto amps = copies ? mps->deep_copy("ARM" + to_string(a)) : mps;
        js << (a ? ", " : "");
        // "DEVICE[:FORM][/SWEEPS][@END][%TOL]": an arm may run fewer sweeps
        // than --sweeps, may stop its forward sweeps at site END (a partial
        // sweep over sites 0 .. END-2, block2's sweep_end_site) and may use
        // its own Davidson tolerance
        string arm = o.arms[a];
        Schedule sc = o.sched;
        Opts oa = o;
        if (arm.find('%') != string::npos) {
            const double tol = atof(arm.substr(arm.find('%') + 1).c_str());
            if (!(tol > 0))
                throw runtime_error("arm " + arm + ": the Davidson tolerance after % must be positive");
            sc.dav_thrds.assign(sc.dav_thrds.size(), tol);
            arm = arm.substr(0, arm.find('%'));
        }
        if (arm.find('@') != string::npos)
            oa.end_site = atoi(arm.substr(arm.find('@') + 1).c_str()), arm = arm.substr(0, arm.find('@'));
        if (arm.find('/') != string::npos)
            sc.nsweeps = atoi(arm.substr(arm.find('/') + 1).c_str()), arm = arm.substr(0, arm.find('/'));
        if (oa.end_site > 0 && sc.nsweeps != 1)
            throw runtime_error("a partial-sweep arm (@END) runs one forward sweep");
        solve_stage<S>(pb, amps, arm, sc, oa, true, "ARM" + to_string(a), js);
    }
    js << "]}\n";
    if (!o.json.empty()) {
        ofstream f(o.json);
        f << js.str();
    }
    mps_info->deallocate();
    pb.mpo->deallocate();
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

static vector<string> parse_words(const string &s) {
    vector<string> r;
    stringstream ss(s);
    string x;
    while (getline(ss, x, ','))
        r.push_back(x);
    return r;
}

} // namespace sweep_driver

int main(int argc, char **argv) {
    sweep_driver::Opts o;
    using sweep_driver::parse_list;
    for (int i = 1; i + 1 < argc; i += 2) {
        string k = argv[i], v = argv[i + 1];
        if (k == "--ham") o.ham = v;
        else if (k == "--L") o.L = atoi(v.c_str());
        else if (k == "--t") o.t = atof(v.c_str());
        else if (k == "--U") o.U = atof(v.c_str());
        else if (k == "--sym") o.sym = v;
        else if (k == "--threads") o.nthreads = atoi(v.c_str());
        else if (k == "--nroots") o.nroots = atoi(v.c_str());
        else if (k == "--seed") o.seed = (unsigned)atol(v.c_str());
        else if (k == "--tol") o.tol = atof(v.c_str());
        else if (k == "--json") o.json = v;
        else if (k == "--scratch") o.scratch = v;
        else if (k == "--stack-gb") o.stack_gb = atof(v.c_str());
        else if (k == "--iprint") o.iprint = atoi(v.c_str());
        else if (k == "--start-site") o.start_site = atoi(v.c_str());
        else if (k == "--end-site") o.end_site = atoi(v.c_str());
        else if (k == "--M") o.sched.bond_dims = parse_list(v);
        else if (k == "--sweeps") o.sched.nsweeps = atoi(v.c_str());
        else if (k == "--noises") o.sched.noises = parse_list(v);
        else if (k == "--noise-type") o.noise_type = v;
        else if (k == "--noise-on-device") o.noise_on_device = atoi(v.c_str());
        else if (k == "--pdm") o.pdm = atoi(v.c_str());
        else if (k == "--pdm-on-gpu") o.pdm_on_gpu = atoi(v.c_str());
        else if (k == "--pdm-order") o.pdm_order = atoi(v.c_str());
        else if (k == "--dav") o.sched.dav_thrds = parse_list(v);
        else if (k == "--arms") o.arms = sweep_driver::parse_words(v);
        else if (k == "--warm-M") o.warm.bond_dims = parse_list(v);
        else if (k == "--warm-sweeps") o.warm.nsweeps = atoi(v.c_str());
        else if (k == "--warm-noises") o.warm.noises = parse_list(v);
        else if (k == "--warm-dav") o.warm.dav_thrds = parse_list(v);
        else if (k == "--warm-device") o.warm_device = v;
        else if (k == "--dump-heff") o.dump_dir = v;
        else if (k == "--dump-arm") o.dump_arm = atoi(v.c_str());
        else if (k == "--dump-sweep") o.dump_sweep = atoi(v.c_str());
        else if (k == "--dump-site") o.dump_site = atoi(v.c_str());
        else {
            cerr << "unknown option " << k << endl;
            return 2;
        }
    }
    if (o.seed == 0) {
        cerr << "--seed must be non-zero (block2 seeds from the clock when given 0)" << endl;
        return 2;
    }
    try {
        if (o.sym == "su2")
            return sweep_driver::run<SU2>(o);
        else if (o.sym == "sz")
            return sweep_driver::run<SZ>(o);
    } catch (const std::exception &ex) {
        cerr << "dmrg_sweep: " << ex.what() << endl;
        return 1;
    }
    cerr << "unknown symmetry " << o.sym << endl;
    return 2;
}
