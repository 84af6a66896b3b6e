"""H_eff*psi and Davidson on the GPU through the C ABI, against the
reference's own outputs (tests/golden) and the oracle."""
import numpy as np
import pytest

from conftest import fixture_ids

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import b2g  # noqa: E402
from oracle import oracle  # noqa: E402

RTOL_FP64 = 1e-12   # plain FP64 H_eff*psi vs the reference, relative 2-norm


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = b2g.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def heffs(ctx, problems):
    hs = {k: b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
          for k, p in problems.items()}
    yield hs
    for h in hs.values():
        h.close()


@pytest.mark.parametrize("name", fixture_ids())
def test_apply_device_matches_reference(problems, heffs, ctx, name):
    p, h = problems[name], heffs[name]
    psi = torch.from_numpy(p.psi).cuda()
    sig = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
    h(psi, sig)
    ctx.synchronize()
    assert rel(sig.cpu().numpy(), p.sigma) <= RTOL_FP64


@pytest.mark.parametrize("name", fixture_ids())
def test_apply_host_matches_reference(problems, heffs, name):
    p, h = problems[name], heffs[name]
    sig = np.zeros(p.sigma_size)
    h(p.psi, sig)
    assert rel(sig, p.sigma) <= RTOL_FP64


@pytest.mark.parametrize("name", fixture_ids())
def test_apply_accumulates_with_scale_and_is_deterministic(problems, heffs, ctx, name):
    p, h = problems[name], heffs[name]
    rng = np.random.default_rng(11)
    x = rng.standard_normal(p.psi_size)
    s0 = rng.standard_normal(p.sigma_size)
    ref = s0 + 0.37 * oracle.replay(p.seq(), p.ops, x, p.sigma_size)
    xs = torch.from_numpy(x).cuda()
    a = torch.from_numpy(s0).cuda()
    b = torch.from_numpy(s0).cuda()
    h(xs, a, 0.37)
    h(xs, b, 0.37)
    ctx.synchronize()
    assert torch.equal(a, b)
    assert rel(a.cpu().numpy(), ref) <= RTOL_FP64


@pytest.mark.parametrize("name", fixture_ids())
def test_davidson_matches_reference(problems, heffs, name):
    p, h = problems[name], heffs[name]
    m = p.meta
    psi = np.array(p.psi, copy=True)
    e, ndav, nflop, tdav = h.eigs(p.diag, psi, conv_thrd=m["conv_thrd"], def_min=m["def_min"],
                                  def_max=m["def_max"])
    assert abs(e + m["const_e"] - m["davidson_energy"]) <= 1e-8
    pf = p.extra["psi_final"]
    assert abs(psi @ pf) / np.linalg.norm(psi) / np.linalg.norm(pf) >= 1 - 1e-6
    assert ndav >= 1 and nflop > 0


RTOL_FP32 = 2e-5    # reduced-precision products (FP32 rounding of operators, W, sums)


@pytest.mark.parametrize("name", fixture_ids())
def test_apply_fp32_form_accuracy(problems, heffs, ctx, name):
    p, h = problems[name], heffs[name]
    psi = torch.from_numpy(p.psi).cuda()
    sig = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
    h(psi, sig, 1.0, b2g.FP32)
    ctx.synchronize()
    assert rel(sig.cpu().numpy(), p.sigma) <= RTOL_FP32


@pytest.mark.parametrize("name", fixture_ids())
def test_davidson_fp32_with_fp64_defect_correction(problems, heffs, name):
    """Basis expanded with FP32 products; convergence declared on FP64
    residuals only; energy = FP64 Rayleigh quotient: within 1e-8 Ha."""
    p, h = problems[name], heffs[name]
    m = p.meta
    psi = np.array(p.psi, copy=True)
    e, ndav, nflop, tdav = h.eigs(p.diag, psi, conv_thrd=m["conv_thrd"], def_min=m["def_min"],
                                  def_max=m["def_max"], form=b2g.FP32)
    r = h.last_davidson
    assert abs(e + m["const_e"] - m["davidson_energy"]) <= 1e-8
    assert r.n_apply_fp64 >= 1 and r.n_apply_mixed >= 1
    assert r.residual_norm2 < m["conv_thrd"]
    # the returned vector's FP64 residual, checked independently on the host
    hx = oracle.replay(p.seq(), p.ops, psi, p.sigma_size)
    lam = psi @ hx / (psi @ psi)
    assert np.sum((hx - lam * psi) ** 2) / (psi @ psi) < 10 * m["conv_thrd"]


RTOL_TF32X3 = 2e-5  # split-TF32 x3 on tensor cores, FP32 accumulation, FP32 work matrices


@pytest.mark.parametrize("name", fixture_ids())
def test_apply_tf32x3_tensor_core_accuracy(problems, heffs, ctx, name):
    p, h = problems[name], heffs[name]
    psi = torch.from_numpy(p.psi).cuda()
    sig = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
    h(psi, sig, 1.0, b2g.TF32X3)
    h.status()
    assert rel(sig.cpu().numpy(), p.sigma) <= RTOL_TF32X3
    # accumulate semantics and determinism (fixed summation order per tile)
    s2 = sig.clone()
    h(psi, s2, -1.0, b2g.TF32X3)
    h.status()
    assert float(torch.max(torch.abs(s2))) <= 1e-12 * float(torch.max(torch.abs(sig)))


@pytest.mark.parametrize("name", fixture_ids())
def test_davidson_tf32x3_with_fp64_defect_correction(problems, heffs, name):
    p, h = problems[name], heffs[name]
    m = p.meta
    psi = np.array(p.psi, copy=True)
    e, ndav, nflop, tdav = h.eigs(p.diag, psi, conv_thrd=m["conv_thrd"], def_min=m["def_min"],
                                  def_max=m["def_max"], form=b2g.TF32X3)
    r = h.last_davidson
    assert abs(e + m["const_e"] - m["davidson_energy"]) <= 1e-8
    assert r.n_apply_mixed >= 1 and r.residual_norm2 < m["conv_thrd"]


def test_size_mismatch_raises(problems, heffs):
    name = sorted(problems)[0]
    h = heffs[name]
    with pytest.raises(ValueError):
        h(np.zeros(h.psi_size + 1), np.zeros(h.sigma_size))


@pytest.mark.parametrize("name", fixture_ids())
@pytest.mark.parametrize("seed", [1, 2])
def test_davidson_from_random_guess_finds_lowest_state(problems, heffs, name, seed):
    """From a random initial guess (the situation of the first sweep from a
    random MPS) both forms converge to the lowest eigenvalue of the symmetric
    H_eff -- the reduced-precision form must not lock onto an excited state
    when its FP64 certifications restart the basis.  Tight threshold 1e-12."""
    p, h = problems[name], heffs[name]
    if p.psi_size != p.sigma_size:
        pytest.skip("bra and ket spaces differ")
    psi0 = np.random.default_rng(seed).standard_normal(p.psi_size)
    out = {}
    for form in (b2g.FP64, b2g.TF32X3):
        x = psi0.copy()
        e, *_ = h.eigs(p.diag, x, conv_thrd=1e-12, form=form)
        out[form] = e
    # the lowest eigenvalue, from a dense FP64 solve of the small H_eff
    ref = min(out.values())
    if p.psi_size <= 4000:
        hm = np.stack([oracle.replay(p.seq(), p.ops, col, p.sigma_size)
                       for col in np.eye(p.psi_size)], axis=1)
        ref = float(np.linalg.eigvalsh(0.5 * (hm + hm.T))[0])
    assert abs(out[b2g.FP64] - ref) <= 1e-8, (out, ref)
    assert abs(out[b2g.TF32X3] - ref) <= 1e-8, (out, ref)
