"""Several right-hand sides at once (state-averaged roots): the batched
H_eff product and the block Davidson, against the single-vector product and
the dense spectrum of the reference's own H_eff."""
import numpy as np
import pytest

from conftest import fixture_ids
from oracle import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import b2g  # noqa: E402

SMALL = [n for n in fixture_ids() if n in ("hub8_su2", "hub8_sz", "syn8_su2", "syn8_sz")]


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = b2g.Context(0)
    yield c
    c.close()


def dense(p):
    """The reference's H_eff as a dense matrix (oracle replay of unit vectors)."""
    n = p.psi_size
    H = np.zeros((n, n))
    e = np.zeros(n)
    for j in range(n):
        e[j] = 1.0
        H[:, j] = oracle.replay(p.seq(), p.ops, e, p.sigma_size)
        e[j] = 0.0
    return H


@pytest.mark.parametrize("name", fixture_ids())
@pytest.mark.parametrize("form,tol", [(b2g.FP64, 1e-12), (b2g.TF32X3, 2e-5)])
def test_apply_batch_equals_single(problems, ctx, name, form, tol):
    p = problems[name]
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    R = 5
    rng = np.random.default_rng(2)
    X = torch.from_numpy(rng.standard_normal((R, p.psi_size))).cuda()
    Y = torch.zeros((R, p.sigma_size), dtype=torch.float64, device="cuda")
    h.apply_batch(X, Y, 0.5, form)
    h.status()
    for r in range(R):
        y = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
        h(X[r].contiguous(), y, 0.5, form)
        h.status()
        ref = 0.5 * oracle.replay(p.seq(), p.ops, X[r].cpu().numpy(), p.sigma_size)
        got = Y[r].cpu().numpy()
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= tol
        if form == b2g.FP64:
            assert torch.equal(Y[r], y)  # same kernels, same order: identical bits
    h.close()


@pytest.mark.parametrize("name", SMALL)
@pytest.mark.parametrize("form", [b2g.FP64, b2g.TF32X3])
def test_block_davidson_four_roots(problems, ctx, name, form):
    p = problems[name]
    w = np.linalg.eigvalsh(0.5 * (lambda H: H + H.T)(dense(p)))
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    k = 4
    rng = np.random.default_rng(4)
    guesses = np.ascontiguousarray(rng.standard_normal((k, p.psi_size)))
    guesses[0] = p.psi
    e, ndav, nflop, tdav = h.eigs_multi(p.diag, guesses, conv_thrd=1e-10, def_min=k, def_max=40, form=form)
    assert np.max(np.abs(e - w[:k])) <= 1e-8, (e, w[:k])
    # eigenvectors: orthonormal, exact residuals small
    G = guesses @ guesses.T
    assert np.allclose(G, np.eye(k), atol=1e-8)
    for i in range(k):
        hx = oracle.replay(p.seq(), p.ops, guesses[i], p.sigma_size)
        assert np.linalg.norm(hx - e[i] * guesses[i]) ** 2 < 1e-9
    h.close()


@pytest.mark.parametrize("name", ["hub16_su2_M250"])
def test_eight_state_averaged_roots_mixed_vs_fp64(problems, ctx, name):
    """Eight roots (the batching form's root count) on the reference's own
    M=250 Hubbard H_eff: the TF32x3 block Davidson with FP64 defect
    correction gives every root energy within 1e-8 of the FP64 block Davidson."""
    p = problems[name]
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    k = 8
    rng = np.random.default_rng(8)
    g0 = np.ascontiguousarray(rng.standard_normal((k, p.psi_size)))
    g0[0] = p.psi
    res = {}
    for form in (b2g.FP64, b2g.TF32X3):
        g = g0.copy()
        e, ndav, nflop, tdav = h.eigs_multi(p.diag, g, conv_thrd=1e-10, def_min=k, def_max=48, form=form)
        res[form] = (e, g)
    e64, etf = res[b2g.FP64][0], res[b2g.TF32X3][0]
    assert np.all(np.diff(e64) >= -1e-12)
    assert np.max(np.abs(etf - e64)) <= 1e-8, (etf, e64)
    h.close()
