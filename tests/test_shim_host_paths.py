"""The shim's host-side translation of block2's PDM expectation products
(GpuTensorFunctions::tensor_product_expectation in b2g_block2.hpp), without a
GPU: the sweep program is built against a stand-in for the library whose
product is the oracle's pair replay (tests/shim_standin.cpp; the host-only
translator b2g_noise_pairs is the library's own source), then block2's
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
    cuda_inc = next((p for p in ("/usr/local/cuda/include", os.path.join(os.environ.get("CUDA_HOME", "/nonexistent"),
                                                                          "include"))
                     if os.path.exists(os.path.join(p, "cuda_runtime.h"))), None)
    if not os.path.exists(os.path.join(BLOCK2, "block2_core.hpp")) or shutil.which("g++") is None or not cuda_inc:
        pytest.skip("block2 headers not staged, no C++ compiler or no CUDA headers")
    d = tmp_path_factory.mktemp("standin")
    exe = str(d / "dmrg_sweep_standin")
    script = f"""
set -e
. "{SHIM}/blas_defs.sh"
gcc -O2 -fopenmp -fPIC -I"{ROOT}/include" -c "{ROOT}/oracle/b2g_oracle.c" -o "{d}/oracle.o"
g++ -std=c++17 -O1 -I"{ROOT}/include" -c "{ROOT}/tests/shim_standin.cpp" -o "{d}/standin.o"
g++ -x c++ -std=c++17 -O1 -I"{cuda_inc}" -I"{ROOT}/include" \\
    -c "{ROOT}/block2-preview_gb300/csrc/b2g_noise.cu" -o "{d}/noise.o"
g++ -std=c++17 -O0 -fopenmp $B2G_BLAS_DEFS -I"{BLOCK2}" -I"{ROOT}/include" -I"{SHIM}" "{SHIM}/dmrg_sweep.cpp" \\
    "{d}/standin.o" "{d}/noise.o" "{d}/oracle.o" -o "{exe}" "$B2G_BLAS" -Wl,-rpath,"$(dirname "$B2G_BLAS")" \\
    -ldl -lpthread
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


@pytest.mark.parametrize("noise_type", ["perturbative", "perturbative-lowmem"])
def test_shim_operator_and_noise_paths_under_block2_davidson(standin_sweep, tmp_path, noise_type):
    """The gpuop arm: block2's own DMRG and host Davidson drive GpuTensorFunctions,
    so every H_eff product goes through the shim's pair translation
    (GpuTensorFunctions::operator()) and every noise product through its
    tensor_product_partial_multiply; with the stand-in's oracle products the
    sweep energies equal block2's CPU arm from the same MPS."""
    js = str(tmp_path / "r.json")
    cmd = [standin_sweep, "--L", "8", "--M", "40", "--sweeps", "4", "--noises", "1e-4,1e-4,1e-5,0", "--dav",
           "1e-10", "--arms", "cpu,cpu,gpuop:fp64", "--threads", "2", "--seed", "1234", "--noise-type",
           noise_type, "--json", js, "--scratch", str(tmp_path / "scr")]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(tmp_path),
                       env=dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    cpu, cpu2, op = json.load(open(js))["arms"]
    spread = np.abs(np.array(cpu["sweep_energies"]) - np.array(cpu2["sweep_energies"]))
    de = np.abs(np.array(op["sweep_energies"]) - np.array(cpu["sweep_energies"]))
    assert np.all(de <= np.maximum(1e-9, 10 * spread)), (de, spread)
    assert op["gpu"]["heff_plans"] > 0 and op["gpu"]["noise_products"] > 0, op["gpu"]


def test_shim_expectation_path_2pdm(standin_sweep, tmp_path):
    """The 2-PDM (PDM2MPOQC: sums of products, many more partials) through the
    drop-in's expectation path equals block2's own 2-PDM of the same MPS."""
    js = str(tmp_path / "r.json")
    cmd = [standin_sweep, "--L", "6", "--M", "30", "--sweeps", "4", "--noises", "1e-4,1e-5,0,0", "--dav", "1e-10",
           "--arms", "cpu", "--threads", "2", "--seed", "1234", "--pdm", "2", "--pdm-on-gpu", "1",
           "--pdm-order", "2", "--json", js, "--scratch", str(tmp_path / "scr")]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(tmp_path),
                       env=dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    arm = json.load(open(js))["arms"][0]
    assert arm["pdm2_device_products"] > 0
    dev, host = np.array(arm["pdm2"]), np.array(arm["pdm2_host"])
    assert dev.size == 6 ** 4 and np.abs(host).max() > 0.1
    assert np.abs(dev - host).max() <= 1e-12, np.abs(dev - host).max()
