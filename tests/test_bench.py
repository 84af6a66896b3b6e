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
