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
