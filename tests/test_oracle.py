"""The oracle (C restatement of the reference's replay and Davidson) pinned
against the reference's own outputs stored in tests/golden."""
import numpy as np
import pytest

from conftest import fixture_ids
from oracle import oracle


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", fixture_ids())
def test_replay_matches_reference_sigma(problems, name):
    p = problems[name]
    s = oracle.replay(p.seq(), p.ops, p.psi, p.sigma_size, nthreads=1)
    assert rel(s, p.sigma) <= 1e-12


@pytest.mark.parametrize("name", fixture_ids())
def test_replay_threads_and_blas(problems, name):
    p = problems[name]
    s1 = oracle.replay(p.seq(), p.ops, p.psi, p.sigma_size, nthreads=4)
    assert rel(s1, p.sigma) <= 1e-12
    if oracle.load_blas():
        s2 = oracle.replay(p.seq(), p.ops, p.psi, p.sigma_size, nthreads=3)
        assert rel(s2, p.sigma) <= 1e-12


@pytest.mark.parametrize("name", fixture_ids())
def test_replay_is_linear(problems, name):
    p = problems[name]
    rng = np.random.default_rng(7)
    x, y = rng.standard_normal(p.psi_size), rng.standard_normal(p.psi_size)
    sx = oracle.replay(p.seq(), p.ops, x, p.sigma_size)
    sy = oracle.replay(p.seq(), p.ops, y, p.sigma_size)
    sxy = oracle.replay(p.seq(), p.ops, 2.0 * x - 0.5 * y, p.sigma_size)
    assert rel(sxy, 2.0 * sx - 0.5 * sy) <= 1e-12


@pytest.mark.parametrize("name", fixture_ids())
def test_heff_symmetric(problems, name):
    """H_eff of a Hermitian Hamiltonian is symmetric: <x|H y> = <y|H x>."""
    p = problems[name]
    rng = np.random.default_rng(3)
    x, y = rng.standard_normal(p.psi_size), rng.standard_normal(p.psi_size)
    hx = oracle.replay(p.seq(), p.ops, x, p.sigma_size)
    hy = oracle.replay(p.seq(), p.ops, y, p.sigma_size)
    assert abs(x @ hy - y @ hx) <= 1e-11 * max(1.0, abs(x @ hy))


@pytest.mark.parametrize("name", fixture_ids())
def test_davidson_matches_reference_energy(problems, name):
    p = problems[name]
    m = p.meta
    e, it, psi, rc = oracle.davidson(p.seq(), p.ops, p.diag, p.psi, m["conv_thrd"],
                                     def_min=m["def_min"], def_max=m["def_max"], nthreads=4)
    assert rc == 0
    assert abs(e + m["const_e"] - m["davidson_energy"]) <= 1e-8
    ov = abs(psi @ p.extra["psi_final"]) / np.linalg.norm(psi) / np.linalg.norm(p.extra["psi_final"])
    assert ov >= 1 - 1e-6


def test_syev_against_numpy():
    rng = np.random.default_rng(1)
    for m in (1, 2, 5, 17, 50):
        a = rng.standard_normal((m, m))
        a = a + a.T
        w, v = oracle.syev(a)
        assert np.allclose(w, np.linalg.eigvalsh(a), atol=1e-11)
        assert np.allclose(a @ v, v * w[None, :], atol=1e-10)
