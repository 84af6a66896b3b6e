"""The shim's host-side translation of block2's PDM expectation products
(GpuTensorFunctions::tensor_product_expectation in b2g_block2.hpp), without a
GPU: the sweep program is built against a stand-in for the library whose
product is the oracle's pair replay (tests/shim_standin.cpp), then block2's
Expect computes the 1-PDM of a converged MPS through the drop-in
(--pdm-on-gpu 1) and with block2's own tensor functions (--pdm 2) on the same
MPS; the two must agree to 1e-12.  Building the program takes about a minute."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SHIM = os.path.join(ROOT, "block2-preview_gb300", "shim")
BLOCK2 = os.path.join(SHIM, "_block2", "src")


@pytest.fixture(scope="module")
def standin_sweep(tmp_path_factory):
    if not os.path.exists(os.path.join(BLOCK2, "block2_core.hpp")) or shutil.which("g++") is None:
        pytest.skip("block2 headers not staged or no C++ compiler")
    d = tmp_path_factory.mktemp("standin")
    exe = str(d / "dmrg_sweep_standin")
    script = f"""
set -e
. "{SHIM}/blas_defs.sh"
gcc -O2 -fopenmp -fPIC -I"{ROOT}/include" -c "{ROOT}/oracle/b2g_oracle.c" -o "{d}/oracle.o"
g++ -std=c++17 -O1 -I"{ROOT}/include" -c "{ROOT}/tests/shim_standin.cpp" -o "{d}/standin.o"
g++ -std=c++17 -O0 -fopenmp $B2G_BLAS_DEFS -I"{BLOCK2}" -I"{ROOT}/include" -I"{SHIM}" "{SHIM}/dmrg_sweep.cpp" \\
    "{d}/standin.o" "{d}/oracle.o" -o "{exe}" "$B2G_BLAS" -Wl,-rpath,"$(dirname "$B2G_BLAS")" \\
    -Wl,--unresolved-symbols=ignore-all -ldl -lpthread
"""
    r = subprocess.run(["bash", "-c", script], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("stand-in build failed:\n" + r.stdout[-3000:] + r.stderr[-3000:])
    return exe


@pytest.mark.parametrize("sym", ["su2", "sz"])
def test_shim_expectation_path_matches_block2(standin_sweep, tmp_path, sym):
    js = str(tmp_path / "r.json")
    cmd = [standin_sweep, "--L", "8", "--M", "40", "--sweeps", "4", "--noises", "1e-4,1e-5,0,0", "--dav", "1e-10",
           "--arms", "cpu", "--threads", "2", "--sym", sym, "--seed", "1234", "--pdm", "2", "--pdm-on-gpu", "1",
           "--json", js, "--scratch", str(tmp_path / "scr")]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(tmp_path),
                       env=dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    arm = json.load(open(js))["arms"][0]
    assert arm["pdm1_device_products"] > 0
    dev, host = np.array(arm["pdm1"]), np.array(arm["pdm1_host"])
    assert np.abs(dev - host).max() <= 1e-12, np.abs(dev - host).max()
    assert abs(np.trace(host.reshape(8, 8)) - 8.0) < 1e-10
