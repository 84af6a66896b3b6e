#!/usr/bin/env python3
"""Benchmark of the two-site DMRG hot path: one H_eff*psi at the middle site.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--form fp64]

A step is one H_eff*psi (sigma = H_eff psi, sigma zeroed first, as the
reference's Davidson does) of the named workload.  `value` is the whole-job
H_eff*psi rate in TFLOP/s (FLOP = 2 x the reference's multiply-add count of
the recorded GEMM pairs) with psi/sigma/operators resident in HBM; `e2e` is
the same rate through the host-buffer C-ABI entry (b2g_heff_apply_host: psi
H2D, product, sigma D2H, inside the timed region).  `--impl reference` times
the CPU restatement of the reference's Tasked replay (BLAS dgemm per pair,
OpenMP over pairs, per-thread sigma copies) on this host's cores.
Multi-GPU: the product does not shard within one H_eff here (replicas only):
each rank runs its own copy and `value` sums the ranks' work over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = ("sweep time & H_eff·ψ TFLOP/s: mixed/batched vs FP64 on 1 GB300 at "
          "|ΔE|≤1e-8 Ha")
L2_BYTES = 129 * 1024 * 1024
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """Samples nvidia-smi clocks / throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None

    def start_time(self):
        return getattr(self, "_t0", None)

    def stop(self):
        if self.proc is None:
            return None
        # nvidia-smi needs a few sampling periods; short timed regions still get samples
        time.sleep(0.7)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in out.strip().splitlines():
            t = [x.strip() for x in ln.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                mx.append(float(t[2]))
            except ValueError:
                continue
            for nm, v in zip(names, t[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- workload
def load_workload(name: str):
    from b2g import workloads
    return workloads.get(name)


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ----------------------------------------------------------------------------- reference arm
def cpu_replay_timing(prob, max_steps: int, budget_s: float, warmup: int = 1):
    """Times the oracle's Tasked replay (reference algorithm, BLAS per pair) with all host threads."""
    from oracle import oracle
    blas = oracle.load_blas()
    nthreads = os.cpu_count() or 1
    seq = prob.seq()
    psi = prob.psi
    for _ in range(max(0, warmup)):
        oracle.replay(seq, prob.ops, psi, prob.sigma_size, nthreads=nthreads)
    times = []
    t_all = time.perf_counter()
    while len(times) < max(1, max_steps):
        t0 = time.perf_counter()
        oracle.replay(seq, prob.ops, psi, prob.sigma_size, nthreads=nthreads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > budget_s:
            break
    return times, nthreads, blas


# ----------------------------------------------------------------------------- our arm
FORMS = {"fp64": 0, "tf32x3": 1, "fp32": 2}
FORM_DTYPE = {"fp64": "f64", "tf32x3": "tf32x3 (split TF32 on tcgen05, f32 accumulate) -> f64 sigma",
              "fp32": "f32 (CUDA cores) -> f64 sigma"}


# measured DRAM traffic of the GEMM0 phase per product (see the roofline note)
G0_TRAFFIC = {"heff_syn24_su2_M1000_sweep0": 1.276e9, "heff_syn24_su2_M1000_mid": 5.35e9}


def workloads_default():
    from b2g import workloads
    return workloads.DEFAULT


def run_ours(args, rank, local_rank, world, dist):
    import ctypes as C

    import torch

    import b2g
    from b2g import capi

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    prob = load_workload(args.workload)
    ctx = b2g.Context(local_rank)
    heff = b2g.EffectiveHamiltonian(ctx, prob.seq(), prob.ops, prob.psi_size, prob.sigma_size)
    st = heff.stats
    # tile shapes of the tensor-core form picked by the autotuner (untimed setup)
    if args.tiles:
        heff.set_params(*[int(x) for x in args.tiles.split(",")])
        tune = None
    else:
        tune = None if args.no_autotune else heff.autotune()
    flop = 2.0 * st["mnk"]
    a = prob.pairs
    flop0 = 2.0 * float(np.sum(a["m0"].astype(np.float64) * a["n0"] * a["k0"]))
    flop1 = 2.0 * float(np.sum(a["m1"].astype(np.float64) * a["n1"] * a["k1"]))
    stream = torch.cuda.ExternalStream(ctx.stream_ptr, device=dev)
    psi = torch.from_numpy(prob.psi).to(dev)
    sig = torch.zeros(prob.sigma_size, dtype=torch.float64, device=dev)
    ws_bytes = st["ops_bytes"] + st["work_bytes"] + 16 * prob.psi_size
    flush = None
    if ws_bytes < 4 * L2_BYTES:
        flush = torch.empty(4 * L2_BYTES, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()

    def do_flush():
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.zero_()

    def step(form):
        with torch.cuda.stream(stream):
            sig.zero_()
        heff.apply_ptr(psi.data_ptr(), sig.data_ptr(), 1.0, form)

    def time_form(form, clocks=None):
        for _ in range(args.warmup):
            step(form)
        heff.status()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        if clocks is not None:
            clocks.start()
        t_wall = time.perf_counter()
        for k in range(args.steps):
            do_flush()
            evs[k][0].record(stream)
            step(form)
            evs[k][1].record(stream)
        heff.status()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
        ck = clocks.stop() if clocks is not None else None
        total = sum(x.elapsed_time(y) for x, y in evs) / 1e3
        # per-kernel times (CUDA events recorded inside the library around each phase)
        capi.check(capi.lib().b2g_heff_set_timing(heff._h, 1))
        ph = []
        for _ in range(3):
            do_flush()
            step(form)
            ms = (C.c_float * 2)()
            capi.check(capi.lib().b2g_heff_last_timing(heff._h, ms))
            ph.append((ms[0], ms[1]))
        capi.check(capi.lib().b2g_heff_set_timing(heff._h, 0))
        p1 = statistics.median(x[0] for x in ph)
        p2 = statistics.median(x[1] for x in ph)
        return total, t_wall, p1, p2, ck, float(torch.linalg.norm(sig))

    head = args.form
    per_form = {}
    head_res = None
    forms_timed = [head] if args.headline_only else [head] + [f for f in FORMS if f != head]
    for name in forms_timed:
        clocks = ClockSampler(local_rank) if name == head else None
        total, t_wall, p1, p2, ck, nrm = time_form(FORMS[name], clocks)
        tt = torch.tensor([total], dtype=torch.float64, device=dev)
        if dist is not None:
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total = float(tt[0])
        per_form[name] = {"value": flop * args.steps * world / total / 1e12, "unit": "TFLOP/s",
                          "ms_per_step": total / args.steps * 1e3,
                          "phase_ms": {"gemm0": p1, "gemm1": p2}}
        if name == head:
            head_res = (total, t_wall, p1, p2, ck, nrm)
    total, t_wall, p1, p2, ck, nrm = head_res
    # sigma of each form against FP64 (relative 2-norm), same psi; every tensor op
    # on the library's stream, synchronized before reading
    with torch.cuda.stream(stream):
        ref = torch.zeros_like(sig)
    heff.apply_ptr(psi.data_ptr(), ref.data_ptr(), 1.0, FORMS["fp64"])
    heff.status()
    for name in forms_timed:
        with torch.cuda.stream(stream):
            out = torch.zeros_like(sig)
        heff.apply_ptr(psi.data_ptr(), out.data_ptr(), 1.0, FORMS[name])
        heff.status()
        with torch.cuda.stream(stream):
            rel = torch.linalg.norm(out - ref) / torch.linalg.norm(ref)
        stream.synchronize()
        per_form[name]["rel_err_vs_fp64"] = float(rel)
    # ---- batched roots (state-averaged form): 8 right-hand sides per launch
    nb = 8
    xb = torch.randn((nb, prob.psi_size), dtype=torch.float64, device=dev)
    yb = torch.zeros((nb, prob.sigma_size), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()  # made on torch's stream, used on the library's
    for name in (() if args.headline_only else ("tf32x3", "fp64")):
        form = FORMS[name]
        for _ in range(2):
            heff.apply_batch(xb, yb, 1.0, form)
        heff.status()
        reps = max(1, args.steps // 4)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            do_flush()
            with torch.cuda.stream(stream):
                yb.zero_()
            heff.apply_batch(xb, yb, 1.0, form)
        e1.record(stream)
        heff.status()
        ms = e0.elapsed_time(e1) / reps
        per_form[name + "_batch8"] = {"value": flop * nb / (ms * 1e-3) / 1e12, "unit": "TFLOP/s",
                                      "ms_per_step": ms, "roots": nb}
    del xb, yb
    # ---- roofline of the dominant kernel of the headline form
    if head == "fp64":
        pk = C.c_double()
        capi.check(capi.lib().b2g_probe_peak(ctx.handle, FORMS["fp64"], C.byref(pk)))
        peak, bound, unit = pk.value, "fp64-pipe", "TFLOP/s"
        peak_src = ("measured in this run: register-resident FP64 FMA loop (b2g_probe_peak); GB300 has "
                    "no FP64 tensor path and MEASURED_PEAKS.json holds no FP64 figure")
        k2 = "simt_phase2<double> (GEMM1 sigma += alpha op(L) W)"
        k1 = "simt_phase1<double> (GEMM0 W = psi op(R))"
    else:
        pk_all = peaks()
        peak = pk_all.get("bf16_tflops", 1900.0)
        bound, unit = "tensor", "TFLOP/s"
        peak_src = ("MEASURED_PEAKS.json bf16_tflops (burst) of measured; dense TF32 is nominally half of "
                    "BF16 and split-TF32x3 issues 3 MMAs per useful product, so 1/6 of this is the "
                    "useful-FLOP ceiling of this kernel")
        if head == "tf32x3":
            k2 = ("g1_kernel + g1_reduce (GEMM1 sigma += alpha op(L) W: bulk-copied TF32 hi/lo "
                  "operand images, tcgen05.mma kind::tf32 x3, TMEM accumulator)")
            k1 = ("g0_pack_psi + g0_kernel (two occupancy classes) (GEMM0 W^T = op(R)^T psi^T, "
                  "tcgen05.mma kind::tf32 x3, epilogue writes the GEMM1 W images)")
        else:
            k2 = "simt_phase2<float> (GEMM1, FP32)"
            k1 = "simt_phase1<float> (GEMM0 W = psi op(R), FP32)"
    if p2 >= p1:
        kname, kflop, kms = k2, flop1, p2
    else:
        kname, kflop, kms = k1, flop0, p1
    achieved = kflop / (kms * 1e-3) / 1e12
    # the split-TF32x3 form issues three TF32 MMAs (half the BF16 rate) per useful
    # product, so its useful-FLOP ceiling is one sixth of the measured BF16 peak
    ceiling = peak / 6.0 if head == "tf32x3" else peak
    # ---- diag(H_eff) from the recorded pairs (once per site in a sweep)
    if not args.headline_only:
        dd = torch.zeros(prob.sigma_size, dtype=torch.float64, device=dev)
        heff.diag(dd)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        heff.diag(dd)
        e1.record(stream)
        torch.cuda.synchronize()
        per_form["diag_ms"] = e0.elapsed_time(e1)
        del dd
    # ---- e2e leg: host buffers through the C-ABI host entry
    form = FORMS[head]
    psi_h = torch.from_numpy(prob.psi).pin_memory().numpy()
    sig_h = torch.zeros(prob.sigma_size, dtype=torch.float64).pin_memory().numpy()
    for _ in range(max(1, args.warmup)):
        sig_h[:] = 0.0
        heff(psi_h, sig_h, 1.0, form)
    e2e_t = []
    if dist is not None:
        dist.barrier()
    for _ in range(args.steps):
        do_flush()
        ctx.synchronize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sig_h[:] = 0.0
        heff(psi_h, sig_h, 1.0, form)
        e2e_t.append(time.perf_counter() - t0)
    tt = torch.tensor([sum(e2e_t)], dtype=torch.float64, device=dev)
    if dist is not None:
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    e2e_total = float(tt[0])
    value = flop * args.steps * world / total / 1e12
    result = {
        "metric": METRIC,
        "value": value,
        "unit": "TFLOP/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": FORM_DTYPE[head],
        "data": prob.meta.get("data", "synthetic"),
        "config": {
            "workload": args.workload,
            "description": prob.meta.get("description", ""),
            "form": head,
            "n_pairs": st["n_pairs"], "n_work_dedup": st["n_work"], "n_sigma_regions": st["n_regions"],
            "mnk": st["mnk"], "mnk_executed": st["mnk_executed"], "psi_size": prob.psi_size,
            "ops_bytes": st["ops_bytes"],
            "l2": "flushed between steps (512 MB write)" if flush is not None else
                  "inputs larger than L2 (operator blob + work > 4x L2)",
            "parallelism": f"replicas x{world}",
            "wall_s_timed_region": t_wall,
            "tile_shapes": heff.params,
            "autotune": tune,
        },
        "forms": per_form,
        "roofline": {
            "bound": bound, "kernel": kname, "achieved": achieved, "peak": peak, "unit": unit,
            "frac": achieved / peak if peak else None, "peak_source": peak_src,
            "frac_of_form_ceiling": achieved / ceiling if ceiling else None,
            "phase_ms": {"gemm0": p1, "gemm1": p2},
            "traffic": G0_TRAFFIC.get(args.workload or workloads_default()) if head == "tf32x3" and kname == k1
            else None,
            "traffic_note": ("DRAM bytes per GEMM0 phase (both g0_kernel classes): ncu dram__bytes_read.sum + "
                             "dram__bytes_write.sum on the sweep-0 site (1.276 GB), scaled to this site by "
                             "the bytes of operator/W images the phase moves (x4.19); "
                             "profiles/g0_g1_kernels_heff_syn24_M1000_sweep0.md"),
        },
        "e2e": {
            "value": flop * args.steps * world / e2e_total / 1e12, "unit": "TFLOP/s",
            "h2d_bytes_per_step": 8 * (prob.psi_size + prob.sigma_size),
            "d2h_bytes_per_step": 8 * prob.sigma_size,
            "ms_per_step": e2e_total / args.steps * 1e3,
        },
        # kernels of ours per apply: TF32x3 g0_pack_psi, two g0_kernel classes, g1_kernel,
        # g1_reduce; FP64 simt_phase1, simt_phase2, simt_reduce; FP32 adds to_float
        "gpu_launches": args.steps * {"tf32x3": 5, "fp64": 3, "fp32": 4}[head],
        "clocks": ck,
        "sigma_norm": nrm,
    }
    # ---- Davidson on a real reference H_eff (Hubbard L=16 U=4 M=250 middle site):
    # plain FP64 vs TF32x3 with FP64 defect correction, energy vs the reference's
    from b2g import workloads
    dprob = workloads.get("heff_hub16_su2_M250")
    dh = b2g.EffectiveHamiltonian(ctx, dprob.seq(), dprob.ops, dprob.psi_size, dprob.sigma_size)
    dav = {"workload": "heff_hub16_su2_M250", "reference_energy": dprob.meta["davidson_energy"],
           "conv_thrd": dprob.meta["conv_thrd"]}
    for name in (() if args.headline_only else ("fp64", "tf32x3")):
        x = np.array(dprob.psi, copy=True)
        e, ndav, nfl, tdav = dh.eigs(dprob.diag, x, conv_thrd=dprob.meta["conv_thrd"],
                                     def_min=dprob.meta["def_min"], def_max=dprob.meta["def_max"],
                                     form=FORMS[name])
        r = dh.last_davidson
        dav[name] = {"energy": e, "abs_err_vs_reference": abs(e + dprob.meta["const_e"]
                                                               - dprob.meta["davidson_energy"]),
                     "iterations": ndav, "fp64_products": r.n_apply_fp64,
                     "reduced_products": r.n_apply_mixed, "seconds": tdav}
    # eight state-averaged roots (the batching form's root count): block
    # Davidson, all new basis vectors of an iteration in one batched product
    if not args.headline_only:
        rng = np.random.default_rng(8)
        g0 = np.ascontiguousarray(rng.standard_normal((8, dprob.psi_size)))
        g0[0] = dprob.psi
        multi = {}
        for name in ("fp64", "tf32x3"):
            g = g0.copy()
            e8, ndav, nfl, tdav = dh.eigs_multi(dprob.diag, g, conv_thrd=dprob.meta["conv_thrd"], def_min=8,
                                                def_max=48, form=FORMS[name])
            r = dh.last_davidson
            multi[name] = {"energies": [float(v) for v in e8], "iterations": ndav,
                           "fp64_products": r.n_apply_fp64, "reduced_products": r.n_apply_mixed,
                           "seconds": tdav}
        multi["max_abs_root_diff_tf32x3_vs_fp64"] = float(
            np.max(np.abs(np.array(multi["tf32x3"]["energies"]) - np.array(multi["fp64"]["energies"]))))
        dav["eight_roots"] = multi
    dh.close()
    result["davidson"] = dav
    # ---- full-size site solve: Davidson FP64 vs TF32x3 + FP64 defect correction
    # on the symmetrised n=24 M=1000 sweep-0 site (200 iterations at most)
    if not args.headline_only:
        result["site_solve"] = {"site": "heff_syn24_su2_M1000_sweep0",
                                **site_solve_section(ctx, load_workload("heff_syn24_su2_M1000_sweep0"))}
    # ---- differentiation form: one adjoint (operator and ket gradients of
    # <x|H_eff|y>, FP64) on this workload, next to the FP64 product
    if not args.headline_only:
        result["adjoint"] = adjoint_section(heff, prob, stream, dev, do_flush, args)
    # ---- density-matrix truncation of the reference's converged psi at the
    # n=24 M=1000 middle site (28 blocks, 2827 states): GPU vs the oracle's
    # numpy/LAPACK restatement, spectrum and discarded weight vs the reference
    if not args.headline_only:
        result["truncation"] = truncation_section(ctx)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        times, nth, blas = cpu_replay_timing(prob, max_steps=10, budget_s=20.0, warmup=1)
        result["cpu_baseline"] = {
            "value": flop / statistics.median(times) / 1e12, "unit": "TFLOP/s", "cores": nth,
            "kind": "port",
            "sample": f"{len(times)} full H_eff*psi products of this workload (median), oracle replay "
                      f"with {'BLAS dgemm' if blas else 'loop'} per pair, {nth} OpenMP threads",
        }
    heff.close()
    ctx.close()
    return result


def adjoint_section(heff, prob, stream, dev, do_flush, args):
    """Time b2g_heff_adjoint (both gradients) and the FP64 product on the same
    H_eff with CUDA events on the library's stream (L2 flushed before each)."""
    import torch

    import b2g
    rng = np.random.default_rng(12)
    x = torch.from_numpy(rng.standard_normal(prob.sigma_size)).to(dev)
    y = torch.from_numpy(prob.psi).to(dev)
    gops = torch.zeros(prob.ops.size, dtype=torch.float64, device=dev)
    gpsi = torch.zeros(prob.psi_size, dtype=torch.float64, device=dev)
    sig = torch.zeros(prob.sigma_size, dtype=torch.float64, device=dev)
    nflop = heff.adjoint_nflop
    torch.cuda.synchronize()
    reps = max(2, min(args.steps, 5))

    def timed(fn):
        fn()
        ts = []
        for _ in range(reps):
            do_flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    ms_adj = timed(lambda: heff.adjoint(x, y, gops, gpsi))
    ms_fwd = timed(lambda: heff.apply_ptr(y.data_ptr(), sig.data_ptr(), 1.0, b2g.FP64))
    return {"form": "fp64", "ms": ms_adj, "tflops": nflop / ms_adj / 1e9,
            "flop": nflop, "fp64_product_ms": ms_fwd,
            "ratio_to_product": ms_adj / ms_fwd,
            "note": "operator gradient + ket gradient of <x|H_eff|y>; median of "
                    f"{reps} after one warm-up, L2 flushed; FP64 DFMA (GB300 has no FP64 tensor path)",
            "integral_gradient": integral_gradient_check(heff.ctx, dev)}


def integral_gradient_check(ctx, dev):
    """dE/dh_pq and dE/d(pq|rs) for every independent integral (36 + 666) at
    the middle site of a converged n=8 SU(2) MPS: the adjoint kernel at the site
    wavefunction, chained through the reference's integral -> operator Jacobian
    at that MPS, against the reference's own 1-/2-PDM elements (fixture made by
    the reference harness)."""
    import torch

    import b2g
    from b2g.autodiff import chain_to_parameters
    from b2g.problem import PAIR_FIELDS
    z = np.load(os.path.join(ROOT, "tests", "golden", "syn8_su2_conv_fullgrad.npz"))
    h = b2g.EffectiveHamiltonian(ctx, b2g.PairSeq({k: z[k] for k in PAIR_FIELDS}), z["ops"],
                                 int(z["psi_size"]), int(z["sigma_size"]))
    v = torch.from_numpy(z["psi"] / np.linalg.norm(z["psi"])).to(dev)
    g = torch.zeros(z["ops"].size, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    h.adjoint(v, v, g, None)
    ctx.synchronize()
    dE = chain_to_parameters(g, z["jac_idx"], z["jac_val"], z["jac_ptr"])
    h.close()
    ref = z["pdm_derivative"]
    big = np.abs(ref) > 1e-3
    return {"workload": "syn8_su2_conv_fullgrad (n=8 SU(2) M=60, converged MPS, middle site, 3250 pairs)",
            "parameters": int(ref.size),
            "norm_rel_err_vs_reference_pdm": float(np.linalg.norm(dE - ref) / np.linalg.norm(ref)),
            "max_rel_err_vs_reference_pdm": float((np.abs(dE - ref) / np.abs(ref))[big].max()),
            "max_abs_err_small_elements": float(np.abs(dE - ref)[~big].max()) if (~big).any() else 0.0,
            "bound": 1e-6}


def site_solve_section(ctx, prob, max_iter=200, conv_thrd=1e-9):
    """Davidson on the full-size site: FP64 against TF32x3 with FP64 defect
    correction.  The recorded structure carries seeded synthetic operator
    values, whose H_eff is not symmetric; the solve runs on (H_eff + H_eff^T)/2,
    one pair sequence of both (b2g PairSeq.symmetrized: the transposed pairs of
    the same blob), so both forms solve the same symmetric problem of the
    site's block structure (twice the pairs of one product)."""
    import b2g
    seq = prob.seq().symmetrized()
    h = b2g.EffectiveHamiltonian(ctx, seq, prob.ops, prob.psi_size, prob.sigma_size)
    h.set_params(256, 256, 64)
    diag = h.diag()
    out = {"workload": "(H + H^T)/2 of the bench workload's H_eff", "pairs": int(seq.n),
           "conv_thrd": conv_thrd, "max_iter": max_iter}
    for name, form in (("fp64", b2g.FP64), ("tf32x3", b2g.TF32X3)):
        x = np.array(prob.psi, copy=True)
        converged = True
        try:
            h.eigs(diag, x, conv_thrd=conv_thrd, max_iter=max_iter, form=form)
        except b2g.B2GError as err:
            if err.code != 5:   # B2G_ERR_NOT_CONVERGED: report the solve as it stopped
                raise
            converged = False
        r = h.last_davidson
        out[name] = {"energy": r.energy, "iterations": r.n_iter, "converged": converged,
                     "fp64_products": r.n_apply_fp64, "reduced_products": r.n_apply_mixed,
                     "seconds": h.last_tdav, "residual_norm2": r.residual_norm2}
    out["abs_energy_diff"] = abs(out["tf32x3"]["energy"] - out["fp64"]["energy"])
    out["speedup_tf32x3_vs_fp64"] = out["fp64"]["seconds"] / out["tf32x3"]["seconds"]
    h.close()
    return out


def adjoint_only(args, local_rank):
    import torch

    import b2g
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    prob = load_workload(args.workload)
    ctx = b2g.Context(local_rank)
    heff = b2g.EffectiveHamiltonian(ctx, prob.seq(), prob.ops, prob.psi_size, prob.sigma_size)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr, device=dev)
    flush = torch.empty(4 * L2_BYTES, dtype=torch.uint8, device=dev)

    def do_flush():
        with torch.cuda.stream(stream):
            flush.zero_()

    res = adjoint_section(heff, prob, stream, dev, do_flush, args)
    heff.close()
    ctx.close()
    return res


def truncation_section(ctx, cpu=True):

    from b2g.truncation import DensityMatrixLayout, split_density_matrix
    path = os.path.join(ROOT, "tests", "golden", "syn24_su2_M1000_dm.npz")
    z = np.load(path)
    lay = DensityMatrixLayout(bool(z["trace_right"]), z["psi_dm"], z["psi_rows"], z["psi_cols"],
                              z["psi_off"], z["dm_dim"])
    k, cut = int(z["bond_dim"]), float(z["cutoff"])
    for _ in range(2):
        res = split_density_matrix(ctx, lay, z["psi"], k, cut)
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        res = split_density_matrix(ctx, lay, z["psi"], k, cut)
        ts.append(time.perf_counter() - t0)
    eig_ref = z["dm_eig"]
    eig = np.concatenate(res.eigenvalues)
    out = {"workload": "syn24_su2_M1000 middle-site density matrix (" + str(int(z["dm_dim"].size))
                       + " blocks, " + str(int(z["dm_dim"].sum())) + " states, largest "
                       + str(int(z["dm_dim"].max())) + ")",
           "gpu_ms": 1e3 * statistics.median(ts), "kept": res.n_kept,
           "error": res.error, "reference_error": float(z["error"]),
           "max_abs_eig_err_vs_reference": float(np.abs(eig - eig_ref).max())}
    if not cpu:
        return out
    from oracle import oracle as _oracle
    t0 = time.perf_counter()
    _oracle.dm_truncate(bool(z["trace_right"]), z["psi_dm"], z["psi_rows"], z["psi_cols"], z["psi_off"],
                        z["dm_dim"], z["psi"], k, cut)
    out["cpu_oracle_ms"] = 1e3 * (time.perf_counter() - t0)
    out["cpu_oracle"] = "numpy (LAPACK syevd) restatement, host threads of the BLAS"
    return out


def run_reference(args):
    prob = load_workload(args.workload)
    flop = 2.0 * prob.mnk
    times, nth, blas = cpu_replay_timing(prob, max_steps=args.steps, budget_s=120.0,
                                         warmup=min(args.warmup, 1))
    v = flop * len(times) / sum(times) / 1e12
    return {
        "metric": METRIC, "value": v, "unit": "TFLOP/s", "impl": "reference", "n_gpus": 0,
        "steps": len(times), "warmup": min(args.warmup, 1), "ms_per_step": sum(times) / len(times) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": prob.meta.get("data", "synthetic"),
        "config": {"workload": args.workload, "form": "fp64", "mnk": prob.mnk, "psi_size": prob.psi_size},
        "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": nth, "kind": "port",
                         "sample": f"{len(times)} H_eff*psi products (of {args.steps} requested, "
                                   f"120 s budget), {'BLAS dgemm' if blas else 'loop'} per pair"},
        "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=None)
    ap.add_argument("--form", default="tf32x3", choices=sorted(FORMS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default tile shapes (no autotuner pass before timing)")
    ap.add_argument("--tiles", default=None,
                    help="tile shapes g0_rows,g1_cols,chunk installed instead of autotuning "
                         "(profiler runs: the autotuner would time candidates under the profiler)")
    ap.add_argument("--truncation-only", action="store_true",
                    help="run only the density-matrix truncation section (GPU, no CPU leg); "
                         "for profiler runs")
    ap.add_argument("--site-solve-only", action="store_true",
                    help="run only the full-size Davidson comparison (FP64 vs TF32x3) on the "
                         "symmetrised workload H_eff")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="run only the differentiation-form section (one FP64 adjoint and one FP64 "
                         "product on the workload); for profiler runs")
    ap.add_argument("--headline-only", action="store_true",
                    help="time only the headline form (no other forms, batched roots or Davidson "
                         "sections); for profiler runs")
    args = ap.parse_args()
    from b2g import workloads
    if args.workload is None:
        args.workload = workloads.DEFAULT
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if args.truncation_only:
        import b2g
        print(json.dumps({"section": "truncation", **truncation_section(b2g.Context(local_rank), cpu=False)}),
              flush=True)
        return
    if args.site_solve_only:
        import b2g
        print(json.dumps({"section": "site_solve",
                          **site_solve_section(b2g.Context(local_rank), load_workload(args.workload))}),
              flush=True)
        return
    if args.adjoint_only:
        print(json.dumps({"section": "adjoint", "workload": args.workload,
                          **adjoint_only(args, local_rank)}), flush=True)
        return
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local_rank)
        td.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        dist = td
    res = run_ours(args, rank, local_rank, world, dist)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
