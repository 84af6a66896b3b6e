#!/usr/bin/env python3
"""Benchmark of the two-site DMRG sweep with the GB300 drop-in under block2.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload syn24|syn16|syn32|hub16] [--fp64-sweeps KF] [--dav THR]

A step is one full two-site sweep of block2's own DMRG::solve at bond
dimension M (all sites, forward), run by the sweep program lib/dmrg_sweep
(block2's DMRG with b2g_block2::GpuTensorFunctions / GpuDMRG installed: every
Davidson solve on the device, block2's environment, truncation and
bookkeeping on the host).  Default workload: the synthetic ab initio
Hamiltonian n=24, N=24, S=0, SU(2), M=1000 (seeded integral recipe).

The state every step starts from: two sweeps at M/4 (mixed form, Davidson
1e-8) from the seeded random MPS.  The step is the first sweep at M from that
MPS: W untimed and then K timed steps each run on their own copy of it
(MPS::deep_copy, one arm of the sweep program each), so every step repeats the
same work, and `--impl reference` times the same sweep with block2's CPU
path.  Mixed form: split-TF32x3 tensor-core products with FP64 defect
correction.  `value` is the mean wall time of the timed steps; block2 drives a
sweep from host memory (every site's operators are uploaded when the sweep
reaches it), so the sweep has no HBM-resident variant and `e2e` is the same
measurement; `device_resident` is the part spent in the device Davidson
solves.  From the same MPS the bench also runs the step in the plain FP64
form (time ratio, |dE|, site by site) and one untimed mixed arm of two sweeps
whose second, the first with M on both sides, gives the steady sweep time and
the middle-site H_eff that is dumped by the drop-in and measured on its own
(H_eff*psi TFLOP/s per form on the real operators, relative error against
FP64, diag(H_eff), both Davidson forms, the roofline of the dominant kernel).

`--impl reference` runs block2's own CPU path (oracle/_ref/dmrg_sweep_ref,
built from block2's sources with no GPU code) on this host's cores: the same
two M/4 sweeps from the same seeded random MPS, then the step, timed (a CPU
sweep takes minutes, so the sample is one step).
Multi-GPU: a sweep does not shard here (replicas only); each rank runs its own
sweep and the slowest rank's time is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = ("sweep time & H_eff·ψ TFLOP/s: mixed/batched vs FP64 on 1 GB300 at "
          "|ΔE|≤1e-8 Ha")
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
# DRAM bytes (read + write, ncu) per algorithmic FLOP of the two TF32x3 product
# phases, captured on the n=24 M=1000 steady middle site: GEMM0 (g0_pack_psi +
# both g0_kernel classes) 18.8 GB for 7.43e11 FLOP, GEMM1 (g1_kernel +
# g1_reduce) 15.8 GB for 1.91e11 FLOP
TRAFFIC_PER_FLOP = {"gemm0": 18.83e9 / 7.429e11, "gemm1": 15.82e9 / 1.911e11}
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "dmrg_sweep_ref")

# name -> Hamiltonian, bond dimension and warm-up noise.
# Warm-up: two sweeps at M/4 (Davidson 1e-8) from the seeded random MPS, then
# sweeps at M, without noise (block2's density-matrix noise at M = 1000
# randomises the kept states for several sweeps).  The reference arm runs the
# same two M/4 sweeps on the host and times the first sweep at M after them,
# which is the first sweep at M of our arm too.
WORKLOADS = {
    "syn24": {"desc": "synthetic ab initio n=24 N=24 S=0 SU(2), M=1000 (integral recipe, numpy default_rng(0))",
              "n": 24, "M": 1000, "sym": "su2", "warm_noises": (0.0,)},
    "syn16": {"desc": "synthetic ab initio n=16 N=16 S=0 SU(2), M=500 (integral recipe, numpy default_rng(0))",
              "n": 16, "M": 500, "sym": "su2", "warm_noises": (0.0,)},
    "syn32": {"desc": "synthetic ab initio n=32 N=32 S=0 SU(2), M=2000 (integral recipe, numpy default_rng(0))",
              "n": 32, "M": 2000, "sym": "su2", "warm_noises": (0.0,), "stack_gb": 48.0},
    "hub16": {"desc": "1D Hubbard L=16 t=1 U=4 OBC half filling S=0 SU(2), M=250",
              "hubbard": True, "n": 16, "M": 250, "sym": "su2", "warm_noises": (1e-6, 1e-7)},
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


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

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.7)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, busy, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in out.strip().splitlines():
            t = [x.strip() for x in ln.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                mx.append(float(t[2]))
                busy.append(float(t[3]))
            except ValueError:
                continue
            for nm, v in zip(names, t[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        # clocks under load: samples above the median power draw
        cut = statistics.median(busy)
        loaded = [s for s, p in zip(sm, busy) if p >= cut] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(busy)}


# ----------------------------------------------------------------------------- helpers
def hamiltonian(spec: dict, workdir: str) -> dict:
    """run_sweep keyword arguments naming the workload's Hamiltonian."""
    from b2g.sweep import fcidump_synthetic
    if spec.get("hubbard"):
        return {"ham": "hubbard", "L": spec["n"], "U": 4.0, "t": 1.0}
    return {"ham": fcidump_synthetic(os.path.join(workdir, "FCIDUMP"), spec["n"], seed=0)}


def host_threads() -> int:
    return len(os.sched_getaffinity(0))


def host_info() -> dict:
    """The host cores block2's CPU path can use and the BLAS it is linked to
    (scipy's bundled LP64 OpenBLAS, as the build recipe resolves it)."""
    import glob
    try:
        import scipy
        libs = sorted(glob.glob(os.path.join(os.path.dirname(scipy.__file__), os.pardir, "scipy.libs",
                                             "libscipy_openblas*.so")))
        blas = os.path.basename(libs[0]) if libs else "not found"
    except ImportError:
        blas = "not found"
    return {"cpu_count": os.cpu_count(), "affinity_cpus": host_threads(), "blas": blas,
            "blas_threads": 1, "openmp_threads": host_threads()}


def rank_device_env(local_rank: int) -> dict:
    """The sweep program uses device 0 of what it sees: give each rank its own GPU."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    devs = vis.split(",") if vis else [str(i) for i in range(local_rank + 1)]
    return {"CUDA_VISIBLE_DEVICES": devs[local_rank]}


def mean(v):
    return float(sum(v) / len(v)) if v else None


def middle_site(rows: list, n_sites: int) -> dict | None:
    """block2's own per-site record of the middle site (sites n/2-1, n/2) of the
    first sweep: Davidson iterations and time, and its multiply-add rate
    (block2 prints 'FLOPS' as multiply-adds per second of the Davidson)."""
    mid = [x for x in rows if x["sweep"] == 0 and x["site"] == n_sites // 2 - 1]
    if not mid:
        return None
    x = mid[0]
    return {"site": x["site"], "ndav": x["ndav"], "tdav_s": x["tdav"], "site_s": x["t"],
            "mnk_per_s": x["mnk_per_s"], "flop_per_s": 2.0 * x["mnk_per_s"]}


def per_site_forms(sites: dict, mixed_tag: str, fp64_tag: str) -> dict:
    """Site by site, the first sweep of the two forms from the same MPS (block2's
    per-site lines): Davidson seconds of each form, the energy difference, and
    the first site where the energies part by more than 1e-9 Ha (from there on
    the two sweeps carry different states)."""
    a = [x for x in sites.get(mixed_tag, []) if x["sweep"] == 0]
    b = [x for x in sites.get(fp64_tag, []) if x["sweep"] == 0]
    rows = [{"site": x["site"], "mixed_tdav": x["tdav"], "fp64_tdav": y["tdav"], "ndav": [x["ndav"], y["ndav"]],
             "dE": x["energy"] - y["energy"]} for x, y in zip(a, b)]
    first = next((r["site"] for r in rows if abs(r["dE"]) > 1e-9), None)
    return {"rows": rows, "first_site_dE_above_1e-9": first,
            "mixed_tdav_sum": sum(r["mixed_tdav"] for r in rows), "fp64_tdav_sum": sum(r["fp64_tdav"] for r in rows)}


def heff_section(dump_dir: str, dev_index: int, reps: int = 5, adjoint: bool = False) -> dict:
    """H_eff*psi on the real middle-site operators the drop-in dumped: each
    form timed with CUDA events on the library's stream (operator blob resident
    in HBM, far above L2), relative error against FP64, per-phase times of the
    mixed form for the roofline, and both Davidson forms on the site."""
    import ctypes as C

    import torch

    import b2g
    from b2g import capi
    from b2g.problem import load_dump
    prob = load_dump(dump_dir)
    ctx = b2g.Context(dev_index)
    dev = torch.device("cuda", dev_index)
    t_plan = time.perf_counter()
    h = b2g.EffectiveHamiltonian(ctx, prob.seq(), prob.ops, prob.psi_size, prob.sigma_size)
    ctx.synchronize()
    t_plan = time.perf_counter() - t_plan
    st = h.stats
    a = prob.pairs
    flop = 2.0 * st["mnk"]
    flop0 = 2.0 * float(np.sum(a["m0"].astype(np.float64) * a["n0"] * a["k0"]))
    flop1 = 2.0 * float(np.sum(a["m1"].astype(np.float64) * a["n1"] * a["k1"]))
    stream = torch.cuda.ExternalStream(ctx.stream_ptr, device=dev)
    psi = torch.from_numpy(prob.extra.get("psi_converged", prob.psi)).to(dev)
    torch.cuda.synchronize()
    out = {"site": int(prob.meta["site"]), "sweep": int(prob.meta["isweep"]), "n_pairs": st["n_pairs"],
           "mnk": st["mnk"], "mnk_executed": st["mnk_executed"], "ops_bytes": st["ops_bytes"],
           "psi_size": prob.psi_size, "plan_build_and_upload_s": t_plan, "forms": {}}
    # diag(H_eff) from the pairs (the Davidson preconditioner, once per site):
    # CUDA events on the library's stream, median of 5, against the dumped diagonal
    dg = torch.zeros(prob.sigma_size, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()  # dg was made on torch's stream
    h.diag(dg)
    ctx.synchronize()
    evd = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(5)]
    for e0, e1 in evd:
        e0.record(stream)
        h.diag(dg)
        e1.record(stream)
    ctx.synchronize()
    out["diag_ms"] = statistics.median(e0.elapsed_time(e1) for e0, e1 in evd)
    if prob.diag is not None:
        ref_d = torch.from_numpy(np.asarray(prob.diag)).to(dev)
        out["diag_max_rel_err_vs_dump"] = float((dg - ref_d).abs().max() / ref_d.abs().max())
    del dg
    sig = {}
    for name, form in (("fp64", b2g.FP64), ("tf32x3", b2g.TF32X3), ("fp32", b2g.FP32)):
        s = torch.zeros(prob.sigma_size, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        for _ in range(2):
            with torch.cuda.stream(stream):
                s.zero_()
            h.apply_ptr(psi.data_ptr(), s.data_ptr(), 1.0, form)
        h.status()
        n = reps if name != "fp64" else 2
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for e0, e1 in ev:
            with torch.cuda.stream(stream):
                s.zero_()
            e0.record(stream)
            h.apply_ptr(psi.data_ptr(), s.data_ptr(), 1.0, form)
            e1.record(stream)
        h.status()
        torch.cuda.synchronize()
        ms = statistics.median(e0.elapsed_time(e1) for e0, e1 in ev)
        # per-phase times (CUDA events the library records around GEMM0 / GEMM1)
        capi.check(capi.lib().b2g_heff_set_timing(h._h, 1))
        with torch.cuda.stream(stream):
            s.zero_()
        h.apply_ptr(psi.data_ptr(), s.data_ptr(), 1.0, form)
        ph = (C.c_float * 2)()
        capi.check(capi.lib().b2g_heff_last_timing(h._h, ph))
        capi.check(capi.lib().b2g_heff_set_timing(h._h, 0))
        torch.cuda.synchronize()
        sig[name] = s.clone()
        out["forms"][name] = {"ms": ms, "tflops": flop / ms / 1e9, "gemm0_ms": ph[0], "gemm1_ms": ph[1]}
    ref = sig["fp64"]
    for name in sig:
        out["forms"][name]["rel_err_vs_fp64"] = float(torch.linalg.norm(sig[name] - ref) / torch.linalg.norm(ref))
    # FP64 sigma on the host (the CPU replay of the reference algorithm is
    # compared against it at this size)
    out["_fp64_sigma"] = sig["fp64"].cpu().numpy()
    del sig
    # roofline of the dominant kernel phase of the mixed form
    pk = peaks()
    peak = pk.get("bf16_tflops")
    tf = out["forms"]["tf32x3"]
    if tf["gemm0_ms"] >= tf["gemm1_ms"]:
        kname, kflop, kms = ("g0_pack_psi + g0_kernel (GEMM0 W^T = op(R)^T psi^T, tcgen05.mma kind::tf32 x3, "
                             "TMEM accumulator, epilogue writes the GEMM1 W images)"), flop0, tf["gemm0_ms"]
    else:
        kname, kflop, kms = ("g1_kernel + g1_reduce (GEMM1 sigma += alpha op(L) W, bulk-copied TF32 hi/lo "
                             "images, tcgen05.mma kind::tf32 x3)"), flop1, tf["gemm1_ms"]
    achieved = kflop / (kms * 1e-3) / 1e12
    out["roofline"] = {
        "bound": "tensor", "kernel": kname, "achieved": achieved, "unit": "TFLOP/s",
        "peak": peak if peak else 1900.0,
        "peak_source": ("MEASURED_PEAKS.json bf16_tflops (burst), of measured" if peak else
                        "fallback 1.9 PFLOP/s bf16, of fallback"),
        "frac": achieved / (peak if peak else 1900.0),
        "frac_of_form_ceiling": achieved / ((peak if peak else 1900.0) / 6.0),
        "form_ceiling_note": ("dense TF32 runs at half the BF16 rate and split-TF32x3 issues three MMAs per "
                              "useful product: one sixth of the BF16 peak is the useful-FLOP ceiling"),
        "algorithmic_flop": kflop, "ms": kms,
        "traffic": kflop * (TRAFFIC_PER_FLOP["gemm0"] if tf["gemm0_ms"] >= tf["gemm1_ms"] else
                            TRAFFIC_PER_FLOP["gemm1"]),
        "traffic_note": ("DRAM read + write bytes of the phase per product: ncu's dram__bytes_read/write.sum "
                         "per algorithmic FLOP measured on the n=24 M=1000 steady middle site (99,823 pairs), "
                         "times this site's FLOP"),
    }
    # the FP64 product (simt_phase1/2<double>): the certification product of the
    # mixed Davidson, against the DFMA ceiling measured here (MEASURED_PEAKS has
    # no FP64 figure); executed FLOP after the GEMM0 de-duplication
    dfma = C.c_double(0.0)
    capi.check(capi.lib().b2g_probe_peak(ctx.handle, b2g.FP64, C.byref(dfma)))
    f64 = out["forms"]["fp64"]
    ach64 = 2.0 * st["mnk_executed"] / (f64["ms"] * 1e-3) / 1e12
    out["roofline_fp64"] = {
        "bound": "fp64 pipe", "kernel": "simt_phase1<double> + simt_phase2<double> (FP64 H_eff*psi on DFMA)",
        "achieved": ach64, "unit": "TFLOP/s", "peak": dfma.value,
        "peak_source": "b2g_probe_peak(B2G_FP64): register-resident DFMA loop measured in this run",
        "frac": ach64 / dfma.value if dfma.value > 0 else None, "executed_flop": 2.0 * st["mnk_executed"],
        "ms": f64["ms"],
        "note": ("in a mixed sweep these FP64 products certify each site's Davidson solve (defect "
                 "correction) and take most of its device time at M >= 1000")}
    # Davidson on the site: FP64 against TF32x3 with FP64 defect correction
    conv = min(float(prob.meta.get("conv_thrd", 1e-10)), 1e-12)
    dav = {"conv_thrd": conv}
    for name, form in (("fp64", b2g.FP64), ("tf32x3", b2g.TF32X3)):
        x = np.array(prob.psi, copy=True)
        e, nd, nf, td = h.eigs(prob.diag, x, conv_thrd=conv, form=form)
        r = h.last_davidson
        dav[name] = {"energy": e + float(prob.meta.get("const_e", 0.0)), "iterations": nd,
                     "fp64_products": r.n_apply_fp64, "reduced_products": r.n_apply_mixed, "seconds": td}
    dav["abs_energy_diff"] = abs(dav["tf32x3"]["energy"] - dav["fp64"]["energy"])
    dav["speedup"] = dav["fp64"]["seconds"] / dav["tf32x3"]["seconds"]
    out["davidson"] = dav
    if adjoint:
        out["adjoint"] = adjoint_section(h, prob, ctx, dev, stream)
    h.close()
    ctx.close()
    return out, prob


def adjoint_section(h, prob, ctx, dev, stream, n_dirs: int = 20) -> dict:
    """The differentiation form on the dumped site: one adjoint of
    f = <psi| H_eff(ops) |psi> (operator gradient, FP64) timed with CUDA events,
    and the gradient checked against central differences of f in n_dirs
    random directions of operator space (f is quadratic in the blob, so the
    central difference is exact up to rounding)."""
    import torch
    psi = torch.from_numpy(prob.extra.get("psi_converged", prob.psi)).to(dev)
    psi = psi / torch.linalg.norm(psi)
    ops = torch.from_numpy(prob.ops).to(dev)
    g = torch.zeros_like(ops)
    torch.cuda.synchronize()
    h.adjoint(psi, psi, g, None)
    ctx.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
    for e0, e1 in ev:
        with torch.cuda.stream(stream):
            g.zero_()
        e0.record(stream)
        h.adjoint(psi, psi, g, None)
        e1.record(stream)
    ctx.synchronize()
    ms = statistics.median(e0.elapsed_time(e1) for e0, e1 in ev)
    sig = torch.zeros(prob.sigma_size, dtype=torch.float64, device=dev)

    def f(blob):
        torch.cuda.current_stream(dev).synchronize()  # blob was made on torch's stream
        h.set_ops(blob)
        with torch.cuda.stream(stream):
            sig.zero_()
        h.apply_ptr(psi.data_ptr(), sig.data_ptr(), 1.0, 0)
        ctx.synchronize()
        return float(torch.dot(psi, sig))

    gen = torch.Generator(device=dev).manual_seed(7)
    scale = float(torch.linalg.norm(ops)) / max(1.0, float(ops.numel()) ** 0.5)
    errs = []
    for _ in range(n_dirs):
        d = torch.randn(ops.shape, dtype=torch.float64, device=dev, generator=gen) * scale
        t = 1e-5
        fd = (f(ops + t * d) - f(ops - t * d)) / (2 * t)
        gd = float(torch.dot(g, d))
        errs.append(abs(gd - fd) / max(abs(fd), 1e-300))
    torch.cuda.current_stream(dev).synchronize()
    h.set_ops(ops)
    ctx.synchronize()
    nflop = h.adjoint_nflop
    return {"what": "gradient of <psi|H_eff(ops)|psi> w.r.t. the operator blob (FP64 adjoint kernel)",
            "ms": ms, "flop": nflop, "tflops": nflop / ms / 1e9,
            "fd_directions": n_dirs, "fd_step": 1e-5, "max_rel_err_vs_central_differences": max(errs),
            "bound": 1e-6}


def cpu_port_rate(prob, psi=None, ref_sigma=None, budget_s: float = 25.0):
    """FLOP/s of the CPU restatement of block2's Tasked replay (oracle port:
    BLAS dgemm per pair, OpenMP over pairs, per-thread sigma copies) on one
    product of the dumped site, all host threads; with ref_sigma, also the
    relative difference of its sigma (psi given) from ref_sigma."""
    from oracle import oracle
    blas = oracle.load_blas()
    nth = host_threads()
    seq = prob.seq()
    x = prob.psi if psi is None else psi
    flop = 2.0 * prob.mnk
    times, rel = [], None
    t_all = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        sg = oracle.replay(seq, prob.ops, x, prob.sigma_size, nthreads=nth)
        times.append(time.perf_counter() - t0)
        if rel is None and ref_sigma is not None:
            rel = float(np.linalg.norm(sg - ref_sigma) / np.linalg.norm(sg))
        if time.perf_counter() - t_all > budget_s or len(times) >= 5:
            break
    return flop / statistics.median(times), len(times), nth, blas, rel


def heff_only(dump_dir: str, form_name: str, products: int, dev_index: int) -> dict:
    """A few products of one form on a dumped H_eff (nothing else runs: for
    profiler captures of the product kernels)."""
    import torch

    import b2g
    from b2g.problem import load_dump
    prob = load_dump(dump_dir)
    ctx = b2g.Context(dev_index)
    dev = torch.device("cuda", dev_index)
    h = b2g.EffectiveHamiltonian(ctx, prob.seq(), prob.ops, prob.psi_size, prob.sigma_size)
    form = {"fp64": b2g.FP64, "tf32x3": b2g.TF32X3, "fp32": b2g.FP32}[form_name]
    psi = torch.from_numpy(prob.extra.get("psi_converged", prob.psi)).to(dev)
    sig = torch.zeros(prob.sigma_size, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = {"section": "heff_only", "form": form_name, "n_pairs": h.stats["n_pairs"], "mnk": h.stats["mnk"],
           "ops_bytes": h.stats["ops_bytes"], "psi_size": prob.psi_size}
    if products > 0:
        for _ in range(products):
            h.apply_ptr(psi.data_ptr(), sig.data_ptr(), 1.0, form)
        h.status()
        out["products"] = products
    else:
        # one Davidson solve from the dumped initial guess (its vector kernels
        # run on psi-sized vectors: the memory-bound part of the solve)
        x = np.array(prob.psi, copy=True)
        e, nd, nf, td = h.eigs(prob.diag, x, conv_thrd=1e-12, form=form)
        out.update(davidson_energy=e, iterations=nd, fp64_products=h.last_davidson.n_apply_fp64,
                   reduced_products=h.last_davidson.n_apply_mixed)
    out["wall_s"] = time.perf_counter() - t0
    h.close()
    ctx.close()
    return out


# ----------------------------------------------------------------------------- our arm
def run_ours(args, rank, local_rank, world, dist):
    """One step = the first full sweep at M from the state that two sweeps at
    M/4 leave (the seeded random MPS, Davidson 1e-8): every step (W untimed,
    then K timed) is an arm of the sweep program that starts from its own copy
    of that one MPS (MPS::deep_copy), so each repeats the same work, and
    `--impl reference` times the same sweep of block2's CPU path.  Beside the
    steps, from the same MPS: the FP64 form on the same sweep, and one untimed
    mixed arm of two sweeps whose second (M on both sides) gives the steady
    sweep time and the dumped middle-site H_eff."""
    import torch

    from b2g.sweep import SWEEP_BIN, run_sweep
    torch.cuda.set_device(local_rank)
    spec = WORKLOADS[args.workload]
    wd = tempfile.mkdtemp(prefix="b2g_bench_", dir=args.workdir)
    ham = hamiltonian(spec, wd)
    prep = 2
    wm, wn, wdv = (spec["M"] // 4,) * prep, (spec["warm_noises"][0],) * prep, (1e-8,) * prep
    W, K, kf = max(0, args.warmup), max(1, args.steps), max(0, args.fp64_sweeps)
    steady_sweep = args.dump_arm_sweep if args.dump_arm_sweep >= 0 else 1
    arms = ["gpu:tf32x3/1"] * (W + K)            # W untimed steps, then the K timed ones
    i_fp64 = len(arms)
    arms += ["gpu:fp64/1"] * kf
    i_steady = len(arms)
    arms.append(f"gpu:tf32x3/{steady_sweep + 1}")
    i_part = len(arms)
    if args.partial_end:
        # both forms on one partial forward sweep (sites 0 .. E-2) from the same MPS
        arms += [f"gpu:fp64/1@{args.partial_end}", f"gpu:tf32x3/1@{args.partial_end}"]
    i_tol = len(arms)
    if args.tol_study:
        # both forms again at a tighter Davidson tolerance: how far each form's
        # sweep energy moves with the tolerance alone
        arms += [f"gpu:tf32x3/1%{args.tol_study:g}", f"gpu:fp64/1%{args.tol_study:g}"]
    i_cpu = len(arms)
    if args.cpu_arm:
        arms.append("cpu/1")
    dump = os.path.join(wd, "heff_dump")
    if dist is not None:
        dist.barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    t0 = time.perf_counter()
    r = run_sweep(binary=SWEEP_BIN, sym=spec["sym"], M=(spec["M"],), sweeps=1, noises=(0.0,),
                  dav=(args.dav,), arms=tuple(arms), warm_sweeps=prep, warm_noises=wn, warm_dav=wdv, warm_M=wm,
                  warm_device="gpu:tf32x3", threads=args.threads or host_threads(),
                  workdir=os.path.join(wd, "run"), dump_heff=dump,
                  # the dumped site: the middle of the steady arm's sweep with M
                  # on both sides, or with --partial-end the last site of the
                  # mixed partial sweep
                  dump_arm=i_part + 1 if args.partial_end else i_steady,
                  dump_sweep=0 if args.partial_end else steady_sweep,
                  dump_site=args.partial_end - 2 if args.partial_end else -1,
                  env=rank_device_env(local_rank) if world > 1 else None,
                  stack_gb=spec.get("stack_gb", 4.0), **ham)
    wall = time.perf_counter() - t0
    ck = clocks.stop()
    timed = r["arms"][W:W + K]
    first = timed[0]
    t_sweep = mean([a["sweep_time"][0] for a in timed])
    tt = torch.tensor([t_sweep], dtype=torch.float64, device="cuda")
    if dist is not None:
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    t_sweep = float(tt[0])
    ph = [a["phases"][0] for a in timed]
    steady = r["arms"][i_steady]
    res = {
        "metric": METRIC, "value": t_sweep, "unit": "s/sweep", "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": t_sweep * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "tf32x3 tensor-core products (f32 accumulate) + f64 Davidson, residual and truncation",
        "data": "synthetic: seeded integrals / Hubbard chain, seeded random initial MPS",
        "config": {"workload": f"{args.workload}: full two-site sweep of block2's DMRG::solve, "
                               f"{spec['desc']}", "n_sites": r["n_sites"], "bond_dim": spec["M"],
                   "step": ("the first sweep at M from the MPS two sweeps at M/4 leave; every step starts "
                            "from its own copy of that MPS"),
                   "davidson_conv_thrd": args.dav, "noise": 0.0,
                   "state_preparation": {"M": wm, "noise": wn, "dav": wdv},
                   "host_threads": r["threads"], "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (operator blobs of GBs per site)"},
        "e2e": {"value": t_sweep, "unit": "s/sweep", "h2d_bytes_per_step": mean([p["h2d_bytes"] for p in ph]),
                "d2h_bytes_per_step": mean([p["d2h_bytes"] for p in ph]),
                "note": ("block2 drives the sweep from host memory: each site's operators are uploaded when "
                         "the sweep reaches it, so value and e2e are one measurement (host clock around "
                         "each DMRG::sweep)")},
        "device_resident": {"s_per_sweep": mean([p["gpu_davidson"] for p in ph]),
                            "what": "time inside the device Davidson solves (operators resident in HBM)"},
        "sweep_breakdown_s": {k: mean([p[k] for p in ph]) for k in
                              ("teff", "teig", "tmve", "tdm", "tsplt", "gpu_davidson", "gpu_translate",
                               "gpu_plan_upload")},
        "sweeps": {"mixed": {"seconds": [a["sweep_time"][0] for a in timed],
                             "energies": [a["sweep_energies"][0] for a in timed],
                             "discarded_weights": first["discarded_weights"], "gpu": first.get("gpu")},
                   "untimed_steps_seconds": [a["sweep_time"][0] for a in r["arms"][:W]],
                   "state_preparation_seconds": r["warm"]["sweep_time"],
                   "state_preparation_energies": r["warm"]["sweep_energies"]},
        "steady_sweep": {"seconds": steady["sweep_time"][steady_sweep],
                         "energy": steady["sweep_energies"][steady_sweep],
                         "breakdown_s": {k: steady["phases"][steady_sweep][k] for k in
                                         ("teff", "teig", "tmve", "tsplt", "gpu_davidson", "gpu_plan_upload")},
                         "what": (f"untimed: sweep {steady_sweep} of one more mixed arm from the same MPS, the "
                                  "first with M on both sides (its middle site is the dumped H_eff)")},
        "gpu_launches": int(sum(a["gpu"]["kernel_launches"] for a in timed)),
        "clocks": ck, "wall_s": wall,
    }
    energies = res["sweeps"]["mixed"]["energies"]
    res["sweeps"]["mixed"]["max_energy_spread"] = max(energies) - min(energies)
    if kf > 0:
        fps = r["arms"][i_fp64:i_fp64 + kf]
        t64 = mean([a["sweep_time"][0] for a in fps])
        dE = [abs(a["sweep_energies"][0] - first["sweep_energies"][0]) for a in fps]
        res["sweeps"]["fp64"] = {"seconds": [a["sweep_time"][0] for a in fps],
                                 "energies": [a["sweep_energies"][0] for a in fps],
                                 "discarded_weights": fps[0]["discarded_weights"], "gpu": fps[0].get("gpu")}
        res["forms"] = {"what": "the same step (first sweep at M from the same MPS) in the FP64 form",
                        "mixed_s_per_sweep": t_sweep, "fp64_s_per_sweep": t64, "fp64_over_mixed": t64 / t_sweep,
                        "abs_dE_per_sweep": dE, "max_abs_dE": max(dE), "dE_bound": 1e-8,
                        "first_sweep_sites": per_site_forms(r["sites"], f"ARM{W}", f"ARM{i_fp64}")}
    if args.partial_end:
        f64p, mxp = r["arms"][i_part], r["arms"][i_part + 1]
        res["partial"] = {"what": f"one partial forward sweep (sites 0..{args.partial_end - 2}) of each form "
                                  "from the same MPS",
                          "mixed_s": mxp["sweep_time"][0], "fp64_s": f64p["sweep_time"][0],
                          "fp64_over_mixed": f64p["sweep_time"][0] / mxp["sweep_time"][0],
                          "abs_dE": abs(mxp["sweep_energies"][0] - f64p["sweep_energies"][0]), "dE_bound": 1e-8,
                          "fp64_davidson_s": f64p["phases"][0]["gpu_davidson"],
                          "mixed_davidson_s": mxp["phases"][0]["gpu_davidson"]}
    if args.tol_study:
        tm, tf = r["arms"][i_tol], r["arms"][i_tol + 1]
        res["tolerance_study"] = {
            "dav": args.dav, "tight_dav": args.tol_study,
            "what": ("both forms from the same MPS at the bench tolerance and at a tighter one: the "
                     "mixed-vs-FP64 energy difference at each tolerance, and how far each form's own "
                     "sweep energy moves when only the Davidson tolerance changes"),
            "abs_dE_mixed_vs_fp64_tight": abs(tm["sweep_energies"][0] - tf["sweep_energies"][0]),
            "mixed_tolerance_shift": abs(tm["sweep_energies"][0] - first["sweep_energies"][0]),
            "tight_energies": {"mixed": tm["sweep_energies"][0], "fp64": tf["sweep_energies"][0]},
            "tight_seconds": {"mixed": tm["sweep_time"][0], "fp64": tf["sweep_time"][0]}}
        if kf > 0:
            res["tolerance_study"]["fp64_tolerance_shift"] = abs(r["arms"][i_fp64]["sweep_energies"][0]
                                                                 - tf["sweep_energies"][0])
    if args.cpu_arm:
        cpu = r["arms"][i_cpu]
        res["sweeps"]["cpu"] = {"energies": cpu["sweep_energies"], "seconds": cpu["sweep_time"],
                                "phases": cpu["phases"]}
        res["same_state_cpu"] = {
            "cpu_s_per_sweep": cpu["sweep_time"][0], "mixed_s_per_sweep": t_sweep,
            "cpu_over_mixed": cpu["sweep_time"][0] / t_sweep,
            "abs_dE_mixed_vs_cpu": abs(cpu["sweep_energies"][0] - first["sweep_energies"][0]),
            "what": "block2's CPU path on the same step from the same MPS"}
        if kf > 0:
            res["same_state_cpu"]["abs_dE_fp64_gpu_vs_cpu"] = abs(cpu["sweep_energies"][0]
                                                                  - r["arms"][i_fp64]["sweep_energies"][0])
    # the dumped middle-site H_eff (M on both sides), on its own
    if rank == 0 and not args.no_heff:
        hs, prob = heff_section(dump, local_rank, adjoint=args.adjoint or args.workload == "syn16")
        sigma64 = hs.pop("_fp64_sigma")
        res["heff"] = hs
        res["roofline"] = hs["roofline"]
        res["roofline_fp64"] = hs["roofline_fp64"]
        if world == 1 and not args.no_cpu_baseline:
            rate, nprod, nth, blas, rel = cpu_port_rate(prob, np.asarray(prob.extra.get("psi_converged", prob.psi)),
                                                        sigma64)
            hs["fp64_vs_cpu_replay_rel"] = rel
            hs["fp64_vs_cpu_replay_note"] = ("the plain FP64 product on the GPU against the oracle's CPU replay of "
                                             "block2's Tasked GEMM pairs (pinned to the reference's own sigma on "
                                             "the golden fixtures) on this full-size site")
            src = r["arms"][i_fp64] if kf > 0 else first
            flop_sweep = 2.0 * src["phases"][0]["mnk"]
            host_part = src["sweep_time"][0] - src["phases"][0]["teig"]
            est = flop_sweep / rate + host_part
            res["cpu_baseline"] = {
                "value": est, "unit": "s/sweep", "cores": nth, "kind": "port",
                "sample": (f"{nprod} products of the dumped middle-site H_eff by the oracle's restatement of "
                           f"block2's Tasked replay ({'BLAS dgemm' if blas else 'loop'} per pair, {nth} OpenMP "
                           f"threads): {rate / 1e12:.3f} TFLOP/s; scaled to the step as the FP64 step's "
                           f"Davidson FLOP ({flop_sweep:.3e}) at that rate plus its host-side time "
                           f"({host_part:.1f} s, block2's own code in both)"),
                "cpu_heff_tflops": rate / 1e12, "host": host_info()}
    import shutil
    if args.keep_dump:
        shutil.rmtree(args.keep_dump, ignore_errors=True)
        shutil.copytree(dump, args.keep_dump)
    shutil.rmtree(wd, ignore_errors=True)
    return res


# ----------------------------------------------------------------------------- reference arm
def run_reference(args):
    from b2g.sweep import run_sweep
    spec = WORKLOADS[args.workload]
    if not os.path.exists(REF_BIN):
        return {"impl": "reference", "unavailable": "block2's CPU build (oracle/_ref/dmrg_sweep_ref) is not "
                                                     "built: build() needs block2's headers"}
    wd = tempfile.mkdtemp(prefix="b2g_ref_", dir=args.workdir)
    ham = hamiltonian(spec, wd)
    nth = host_threads()
    t0 = time.perf_counter()
    r = run_sweep(binary=REF_BIN, sym=spec["sym"], M=(spec["M"],), sweeps=1, noises=(0.0,), dav=(args.dav,),
                  arms=("cpu",), warm_sweeps=2, warm_M=(spec["M"] // 4,), warm_noises=(0.0,), warm_dav=(1e-8,),
                  warm_device="cpu", threads=nth, workdir=os.path.join(wd, "run"),
                  stack_gb=spec.get("stack_gb", 4.0), **ham)
    wall = time.perf_counter() - t0
    arm = r["arms"][0]
    v = mean(arm["sweep_time"])
    import shutil
    shutil.rmtree(wd, ignore_errors=True)
    p = arm["phases"][0]
    sample = (f"one step (the first full sweep at M) of block2's CPU DMRG::solve (its OpenMP Tasked GEMM "
              f"replay, scipy's OpenBLAS, {nth} threads) after two sweeps at M/4 from the seeded random MPS, "
              f"Davidson {args.dav:g}; a CPU sweep of this workload takes minutes, so one step is the sample")
    return {
        "metric": METRIC, "value": v, "unit": "s/sweep", "impl": "reference", "n_gpus": 0, "steps": 1,
        "warmup": 0, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic: seeded integrals / Hubbard chain, seeded random initial MPS",
        "config": {"workload": f"{args.workload}: full two-site sweep of block2's DMRG::solve, {spec['desc']}",
                   "n_sites": r["n_sites"], "bond_dim": spec["M"],
                   "step": ("the first sweep at M from the MPS two sweeps at M/4 leave; every step starts "
                            "from its own copy of that MPS"),
                   "davidson_conv_thrd": args.dav, "noise": 0.0,
                   "state_preparation": {"M": (spec["M"] // 4,) * 2, "noise": (0.0,) * 2, "dav": (1e-8,) * 2},
                   "host_threads": nth},
        "cpu_baseline": {"value": v, "unit": "s/sweep", "cores": nth, "kind": "reference", "sample": sample,
                         "host": host_info()},
        "e2e": {"value": v, "unit": "s/sweep", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "phases": {k: p[k] for k in ("teff", "teig", "tmve", "tdm", "tsplt")},
        "middle_site": middle_site(r["sites"].get("ARM0", []), r["n_sites"]),
        "energy": arm["sweep_energies"], "wall_s": wall,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3,
                    help="timed steps: each the first sweep at M from the prepared MPS, mixed form")
    ap.add_argument("--warmup", type=int, default=3, help="untimed steps before the timed ones")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="syn24", choices=sorted(WORKLOADS))
    ap.add_argument("--fp64-sweeps", type=int, default=1,
                    help="the same step in the plain FP64 form, this many times (for the ratio)")
    ap.add_argument("--dav", type=float, default=1e-12, help="Davidson threshold of the timed sweeps")
    ap.add_argument("--threads", type=int, default=0, help="host threads of block2 (default: all)")
    ap.add_argument("--partial-end", type=int, default=0,
                    help="compare the forms on one partial forward sweep ending at this site")
    ap.add_argument("--cpu-arm", action="store_true",
                    help="also run one sweep of block2's CPU path from the same warmed MPS")
    ap.add_argument("--tol-study", type=float, default=0.0, metavar="TOL",
                    help="also run both forms from the same MPS with Davidson threshold TOL")
    ap.add_argument("--no-heff", action="store_true", help="skip the dumped-site H_eff measurements")
    ap.add_argument("--adjoint", action="store_true",
                    help="time the adjoint on the dumped site and check it against central differences "
                         "(always on for syn16, the differentiation form's configuration)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workdir", default=None)
    ap.add_argument("--dump-arm-sweep", type=int, default=-1, metavar="S",
                    help="measure the middle-site H_eff of sweep S of the untimed steady arm (default 1, the "
                         "first with M on both sides)")
    ap.add_argument("--keep-dump", default=None,
                    help="copy the dumped middle-site H_eff to this directory (for --heff-only runs)")
    ap.add_argument("--heff-only", default=None, metavar="DUMP",
                    help="only time H_eff*psi products of a dumped H_eff (profiler runs)")
    ap.add_argument("--form", default="tf32x3", choices=["fp64", "tf32x3", "fp32"],
                    help="--heff-only: the form to run")
    ap.add_argument("--products", type=int, default=3,
                    help="--heff-only: products to run (0: one Davidson solve instead)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    if args.heff_only:
        print(json.dumps(heff_only(args.heff_only, args.form, args.products, local_rank)), flush=True)
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
