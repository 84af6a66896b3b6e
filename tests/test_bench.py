"""bench.py's contract on the CPU: it parses, and its reference arm (block2's
own CPU sweep, built from block2's sources) prints one JSON line with the
keys the bench contract asks for, on the small Hubbard workload."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "dmrg_sweep_ref")


def test_bench_compiles():
    with open(os.path.join(ROOT, "bench.py")) as f:
        compile(f.read(), "bench.py", "exec")


@pytest.mark.skipif(not os.path.exists(REF_BIN), reason="block2 reference build absent")
def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "hub16"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "impl", "higher_is_better", "cpu_baseline", "e2e", "config"):
        assert k in line
    assert line["impl"] == "reference" and line["unit"] == "s/sweep" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "reference"
    # one sweep at M after two at M/4: variational, above the converged
    # Hubbard L=16 U=4 M=250 energy and well below the random start
    assert -8.818767454782 - 1e-8 < line["energy"][-1] < -8.0
    # block2's own record of the middle site and the host the sweep ran on
    assert line["middle_site"]["site"] == 7 and line["middle_site"]["flop_per_s"] > 0
    assert line["cpu_baseline"]["host"]["affinity_cpus"] >= 1


def test_bench_site_helpers():
    """The per-site form comparison and block2's middle-site record, read from
    block2's own per-site lines (the format DMRG::sweep prints at iprint 2)."""
    sys.path.insert(0, ROOT)
    import bench
    from b2g.sweep import parse_sites
    out = "\n".join([
        "== stage ARM0: gpu:tf32x3, 1 sweeps",
        "Sweep =    0 | Direction =  forward | Bond dimension = 1000",
        " --> Site =    0-   1 .. Mmps =    3 Ndav =   2 E =   -10.0000000000 Error = 0.00e+00 "
        "FLOPS = 1.00e+09 Tdav = 0.01 T = 0.02",
        " --> Site =    1-   2 .. Mmps =   10 Ndav =   5 E =   -10.5000000000 Error = 1.00e-14 "
        "FLOPS = 2.00e+12 Tdav = 0.50 T = 0.70",
        "== stage ARM1: gpu:fp64, 1 sweeps",
        "Sweep =    0 | Direction =  forward | Bond dimension = 1000",
        " --> Site =    0-   1 .. Mmps =    3 Ndav =   2 E =   -10.0000000000 Error = 0.00e+00 "
        "FLOPS = 1.00e+09 Tdav = 0.02 T = 0.03",
        " --> Site =    1-   2 .. Mmps =   10 Ndav =   4 E =   -10.5000000100 Error = 1.00e-14 "
        "FLOPS = 2.00e+11 Tdav = 4.00 T = 4.20",
    ])
    sites = parse_sites(out)
    f = bench.per_site_forms(sites, "ARM0", "ARM1")
    assert [r["site"] for r in f["rows"]] == [0, 1]
    assert f["first_site_dE_above_1e-9"] == 1
    assert abs(f["rows"][1]["dE"] - 1e-8) < 1e-12 and f["fp64_tdav_sum"] == 4.02
    m = bench.middle_site(sites["ARM0"], 4)
    assert m["site"] == 1 and m["ndav"] == 5 and m["flop_per_s"] == 4.0e12


def test_bench_step_bookkeeping(monkeypatch):
    """run_ours on a stand-in sweep program: the arm list (W untimed steps, K
    timed steps, the FP64 step, the steady arm, optional arms), which arm's
    sweep is dumped, and which arms feed `value`, `forms` and the optional
    sections.  No GPU: torch's device calls and the sweep program are replaced."""
    import argparse

    import torch
    sys.path.insert(0, ROOT)
    import bench
    import b2g.sweep as sw
    seen = {}

    def fake_run_sweep(**kw):
        arms = kw["arms"]
        seen.update(arms=arms, dump_arm=kw["dump_arm"], dump_sweep=kw["dump_sweep"])
        out = {"n_sites": 24, "threads": 8, "warm": {"sweep_time": [1.0, 1.0], "sweep_energies": [-1.0, -2.0]},
               "arms": [], "sites": {}}
        for i, a in enumerate(arms):
            n = int(a.split("/")[1].split("@")[0].split("%")[0]) if "/" in a else 1
            ph = {k: 0.1 for k in ("teff", "teig", "tmve", "tdm", "tsplt", "gpu_davidson", "gpu_translate",
                                   "gpu_plan_upload", "mnk", "h2d_bytes", "d2h_bytes")}
            out["arms"].append({"sweep_time": [10.0 + i] * n, "sweep_energies": [-3.0 - 1e-10 * i] * n,
                                "discarded_weights": [0.0] * n, "phases": [dict(ph) for _ in range(n)],
                                "gpu": {"kernel_launches": 5}})
        return out

    monkeypatch.setattr(sw, "run_sweep", fake_run_sweep)
    monkeypatch.setattr(torch.cuda, "set_device", lambda *a, **k: None)
    real_tensor = torch.tensor
    monkeypatch.setattr(torch, "tensor", lambda *a, **k: real_tensor(*a, **{x: y for x, y in k.items()
                                                                            if x != "device"}))
    monkeypatch.setattr(bench.ClockSampler, "start", lambda self: None)
    monkeypatch.setattr(bench.ClockSampler, "stop", lambda self: {"sm_mhz": 1.0})
    ns = argparse.Namespace(workload="syn24", warmup=2, steps=3, fp64_sweeps=1, dump_arm_sweep=-1, partial_end=0,
                            tol_study=1e-13, cpu_arm=True, workdir=None, dav=1e-12, threads=0, no_heff=True,
                            keep_dump=None, adjoint=False, no_cpu_baseline=True)
    res = bench.run_ours(ns, 0, 0, 1, None)
    assert seen["arms"] == ("gpu:tf32x3/1",) * 5 + ("gpu:fp64/1", "gpu:tf32x3/2", "gpu:tf32x3/1%1e-13",
                                                     "gpu:fp64/1%1e-13", "cpu/1")
    assert (seen["dump_arm"], seen["dump_sweep"]) == (6, 1)      # the steady arm's second sweep
    assert res["steps"] == 3 and res["warmup"] == 2
    assert res["value"] == 13.0                                   # arms 2..4: 12, 13, 14 s
    assert res["sweeps"]["untimed_steps_seconds"] == [10.0, 11.0]
    assert res["forms"]["fp64_s_per_sweep"] == 15.0 and res["steady_sweep"]["seconds"] == 16.0
    assert res["tolerance_study"]["tight_seconds"] == {"mixed": 17.0, "fp64": 18.0}
    assert res["same_state_cpu"]["cpu_s_per_sweep"] == 19.0
    assert res["gpu_launches"] == 15
    # the partial-sweep comparison dumps the last site of its mixed partial arm
    ns.partial_end, ns.tol_study, ns.cpu_arm = 10, 0.0, False
    res = bench.run_ours(ns, 0, 0, 1, None)
    assert seen["arms"][-2:] == ("gpu:fp64/1@10", "gpu:tf32x3/1@10")
    assert (seen["dump_arm"], seen["dump_sweep"]) == (8, 0)
    assert res["partial"]["fp64_s"] == 17.0 and res["partial"]["mixed_s"] == 18.0
