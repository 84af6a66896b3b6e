import glob
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_NO_GPU = None


def _no_gpu_here():
    """True only on a machine with no NVIDIA device at all: torch sees no CUDA
    device and no NVIDIA device node exists."""
    global _NO_GPU
    if _NO_GPU is None:
        nodes = ("/dev/nvidiactl", "/dev/nvidia0", "/dev/nvidia-uvm")
        try:
            import torch
            visible = torch.cuda.is_available()
        except Exception:
            visible = False
        _NO_GPU = not visible and not any(os.path.exists(n) for n in nodes)
    return _NO_GPU


def pytest_runtest_setup(item):
    """GPU tests are skipped on a machine with no NVIDIA device; wherever a
    device is present they run, and fail loudly if CUDA does not work."""
    if item.get_closest_marker("gpu") is not None and _no_gpu_here():
        pytest.skip("no NVIDIA device on this machine")


def fixture_paths():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def all_ids():
    return [os.path.basename(p)[:-4] for p in fixture_paths()]


def fixture_ids():
    """Effective-Hamiltonian problems (H_eff*psi and Davidson)."""
    return [n for n in all_ids() if not n.endswith(("_rot", "_dm", "_blk", "_qn", "_grad", "_fullgrad", "_cinfo",
                                                     "_effprob", "_noise", "_npdm"))]


def noise_ids():
    """Perturbative-noise products (single-GEMM lists, tests/golden/make_noise_fixtures.py)."""
    return [n for n in all_ids() if n.endswith("_noise")]


def npdm_ids():
    """One site of the reference's PDM expectation sweep (tests/golden/make_npdm_fixtures.py)."""
    return [n for n in all_ids() if n.endswith("_npdm")]


def rotation_ids():
    """Operator-rotation problems (same pair format, no Davidson)."""
    return [n for n in all_ids() if n.endswith("_rot")]


@pytest.fixture(scope="session")
def problems():
    from b2g.problem import load_problem
    return {os.path.basename(p)[:-4]: load_problem(p) for p in fixture_paths()
            if not p.endswith(("_dm.npz", "_blk.npz", "_qn.npz", "_grad.npz", "_fullgrad.npz", "_cinfo.npz",
                               "_effprob.npz", "_noise.npz", "_npdm.npz"))}
