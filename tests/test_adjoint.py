"""Differentiation form: the adjoint of H_eff*psi.

CPU: the numpy adjoint (oracle.adjoint) equals directional derivatives of the
oracle replay, which is pinned to the reference's sigma; the H_eff of every
fixture is symmetric.  GPU: b2g_heff_adjoint equals the oracle adjoint, is
deterministic, and the autograd functions (b2g.autodiff) agree with central
finite differences -- of <x|H|y> in random directions of (ops, psi), and of
the converged lowest eigenvalue in 20 random operator directions (relative
error <= 1e-6).  H_eff is quadratic in the operator blob (each pair multiplies
a left and a right operator block), so central differences of <x|H|y> are
exact up to rounding."""
import numpy as np
import pytest

from conftest import fixture_ids, rotation_ids
from oracle import oracle

RTOL_ADJ = 1e-12      # GPU adjoint vs the numpy adjoint, relative 2-norm
RTOL_FD_LINEAR = 1e-10
RTOL_FD_EIG = 1e-6    # converged-energy derivative vs central differences (step 1e-5)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _rand_like(rng, n, scale=1.0):
    return rng.standard_normal(n) * scale


# ---------------------------------------------------------------- CPU (oracle)

@pytest.mark.parametrize("name", fixture_ids() + rotation_ids())
def test_oracle_adjoint_is_the_derivative_of_the_replay(problems, name):
    p = problems[name]
    seq = p.seq()
    rng = np.random.default_rng(5)
    x = _rand_like(rng, p.sigma_size)
    y = _rand_like(rng, p.psi_size)
    gops, gy = oracle.adjoint(seq, p.ops, x, y)
    # f(ops, y) = x . replay(ops, y) is linear in y and quadratic in ops (each
    # pair multiplies two blocks of the blob), so central differences of any
    # step are exact directional derivatives in ops, and replays of the
    # direction itself are exact in y
    f = lambda o: float(x @ oracle.replay(seq, o, y, p.sigma_size))  # noqa: E731
    for _ in range(3):
        d_ops = _rand_like(rng, p.ops.size)
        d_y = _rand_like(rng, p.psi_size)
        f_ops = 0.5 * (f(p.ops + d_ops) - f(p.ops - d_ops))
        f_y = float(x @ oracle.replay(seq, p.ops, d_y, p.sigma_size))
        assert float(gops @ d_ops) == pytest.approx(f_ops, rel=RTOL_FD_LINEAR, abs=1e-12)
        assert float(gy @ d_y) == pytest.approx(f_y, rel=RTOL_FD_LINEAR, abs=1e-12)


@pytest.mark.parametrize("name", fixture_ids() + rotation_ids())
def test_transposed_pairs_apply_the_transpose(problems, name):
    """PairSeq.transposed(): its replay is H^T x (the adjoint's ket gradient);
    symmetrized() replays (H + H^T)/2 (square problems)."""
    p = problems[name]
    seq = p.seq()
    rng = np.random.default_rng(4)
    x, y = _rand_like(rng, p.sigma_size), _rand_like(rng, p.psi_size)
    _, gy = oracle.adjoint(seq, p.ops, x, y)
    assert rel(oracle.replay(seq.transposed(), p.ops, x, p.psi_size), gy) <= 1e-12
    if p.psi_size == p.sigma_size:
        hs = oracle.replay(seq.symmetrized(), p.ops, x, p.sigma_size)
        ref = 0.5 * (oracle.replay(seq, p.ops, x, p.sigma_size) + gy)
        assert rel(hs, ref) <= 1e-12


@pytest.mark.parametrize("name", fixture_ids())
def test_heff_is_symmetric(problems, name):
    """<x|H y> = <H x|y> on every recorded H_eff (the adjoint's ket gradient is H^T x)."""
    p = problems[name]
    seq = p.seq()
    rng = np.random.default_rng(6)
    x, y = _rand_like(rng, p.sigma_size), _rand_like(rng, p.psi_size)
    _, gy = oracle.adjoint(seq, p.ops, x, y)
    hx = oracle.replay(seq, p.ops, x, p.sigma_size)
    assert rel(gy, hx) <= 1e-12


def _grad_fixture(name="syn8_su2_s0_grad"):
    import json
    import os
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


RTOL_INTEGRAL = 1e-6   # dE/dh_pq, dE/d(pq|rs) vs the reference's own central differences


def _check_integral_gradient(dE, z, meta):
    fd = (z["e_plus"] - z["e_minus"]) / (2 * meta["delta"])
    err = np.abs(dE - fd) / np.abs(fd)
    assert err.max() <= RTOL_INTEGRAL, list(zip(meta["labels"], err))


def test_oracle_integral_gradient_matches_reference_differences():
    """dE/dtheta for one-electron h_pq and two-electron (pq|rs) elements at the
    first site of the first sweep: the numpy adjoint at the reference's
    converged eigenvector, chained through the reference's integral -> operator
    Jacobian, equals the reference's central differences of its own energies."""
    from b2g.autodiff import chain_to_parameters
    from b2g.capi import PairSeq
    from b2g.problem import PAIR_FIELDS
    z, meta = _grad_fixture()
    seq = PairSeq({k: z[k] for k in PAIR_FIELDS})
    v = z["psi_final"] / np.linalg.norm(z["psi_final"])
    g, _ = oracle.adjoint(seq, z["ops"], v, v)
    dE = chain_to_parameters(g, z["jac_idx"], z["jac_val"], z["jac_ptr"])
    _check_integral_gradient(dE, z, meta)


def _check_pdm_derivative(dE, z, meta):
    ref = z["pdm_derivative"]
    err = np.abs(dE - ref) / np.abs(ref)
    assert err.max() <= RTOL_INTEGRAL, list(zip(meta["labels"], err))


def test_oracle_integral_gradient_matches_reference_pdm():
    """At a converged MPS (fixed), dE/dh_pq and dE/d(pq|rs) from the numpy
    adjoint at the MPS centre, chained through the reference's integral ->
    operator Jacobian at that MPS, equal the reference's own 1-/2-PDM elements
    (Expect; E = sum h dm1 + 1/2 sum (ij|kl) dm2[i,k,l,j], checked when the
    fixture was made)."""
    from b2g.autodiff import chain_to_parameters
    from b2g.capi import PairSeq
    from b2g.problem import PAIR_FIELDS
    z, meta = _grad_fixture("syn8_su2_conv_grad")
    seq = PairSeq({k: z[k] for k in PAIR_FIELDS})
    v = z["psi"] / np.linalg.norm(z["psi"])
    g, _ = oracle.adjoint(seq, z["ops"], v, v)
    _check_pdm_derivative(chain_to_parameters(g, z["jac_idx"], z["jac_val"], z["jac_ptr"]), z, meta)


def _check_full_gradient(dE, ref):
    """Every independent integral: per-element relative error <= 1e-6 where the
    PDM element exceeds 1e-3, absolute <= 1e-9 elsewhere."""
    big = np.abs(ref) > 1e-3
    assert np.all(np.abs(dE - ref)[big] / np.abs(ref[big]) <= RTOL_INTEGRAL)
    assert np.all(np.abs(dE - ref)[~big] <= 1e-9)


def _jac_times(z, d):
    """sum_k d_k dops/dtheta_k (the blob is linear in the integrals)."""
    ptr = z["jac_ptr"]
    col = np.repeat(np.arange(ptr.size - 1), np.diff(ptr))
    out = np.zeros(z["ops"].size)
    np.add.at(out, z["jac_idx"], z["jac_val"] * d[col])
    return out


def test_oracle_full_integral_gradient_matches_reference_pdm():
    """dE/dh_pq and dE/d(pq|rs) for every independent integral (36 + 666 at n=8)
    at the converged MPS: numpy adjoint chained through the reference's full
    Jacobian, against the reference's 1-/2-PDM."""
    from b2g.autodiff import chain_to_parameters
    from b2g.capi import PairSeq
    from b2g.problem import PAIR_FIELDS
    z, meta = _grad_fixture("syn8_su2_conv_fullgrad")
    assert len(meta["labels"]) == 702
    seq = PairSeq({k: z[k] for k in PAIR_FIELDS})
    v = z["psi"] / np.linalg.norm(z["psi"])
    g, _ = oracle.adjoint(seq, z["ops"], v, v)
    _check_full_gradient(chain_to_parameters(g, z["jac_idx"], z["jac_val"], z["jac_ptr"]),
                         z["pdm_derivative"])


# ---------------------------------------------------------------- GPU

torch = pytest.importorskip("torch")
import b2g  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = b2g.Context(0)
    yield c
    c.close()


def _heff(ctx, p):
    return b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)


@pytest.mark.gpu
@pytest.mark.parametrize("name", fixture_ids() + rotation_ids())
def test_gpu_adjoint_matches_oracle_and_is_deterministic(problems, ctx, name):
    p = problems[name]
    h = _heff(ctx, p)
    rng = np.random.default_rng(7)
    x = _rand_like(rng, p.sigma_size)
    y = _rand_like(rng, p.psi_size)
    ref_ops, ref_y = oracle.adjoint(p.seq(), p.ops, x, y)
    xd, yd = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    outs = []
    for _ in range(2):
        gops = torch.zeros(p.ops.size, dtype=torch.float64, device="cuda")
        gy = torch.zeros(p.psi_size, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        h.adjoint(xd, yd, gops, gy, scale=0.5)
        ctx.synchronize()
        outs.append((gops.cpu().numpy(), gy.cpu().numpy()))
    assert rel(outs[0][0], 0.5 * ref_ops) <= RTOL_ADJ
    assert rel(outs[0][1], 0.5 * ref_y) <= RTOL_ADJ
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert h.adjoint_nflop > 0
    h.close()


@pytest.mark.gpu
def test_set_ops_updates_every_form(problems, ctx):
    p = problems["hub16_su2_M250"]
    h = _heff(ctx, p)
    psi = torch.from_numpy(p.psi).cuda()
    for form, tol in ((b2g.FP64, 1e-12), (b2g.TF32X3, 1e-4)):
        s1 = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        h(psi, s1, form=form)
        h.set_ops(2.0 * p.ops)          # host values (every pair multiplies two blocks: 4 sigma)
        s2 = torch.zeros_like(s1)
        torch.cuda.synchronize()
        h(psi, s2, form=form)
        h.set_ops(torch.from_numpy(p.ops).cuda())   # device values
        s3 = torch.zeros_like(s1)
        torch.cuda.synchronize()
        h(psi, s3, form=form)
        ctx.synchronize()
        a, b, c = s1.cpu().numpy(), s2.cpu().numpy(), s3.cpu().numpy()
        assert rel(b, 4.0 * a) <= tol
        assert rel(c, a) <= tol
        assert rel(a, p.sigma) <= tol
    h.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", fixture_ids())
def test_autograd_matches_finite_differences(problems, ctx, name):
    """d<x|H(ops)|y> by torch.autograd through HeffApply vs central differences
    in random directions of ops and psi."""
    from b2g.autodiff import heff_apply
    p = problems[name]
    h = _heff(ctx, p)
    rng = np.random.default_rng(8)
    ops = torch.from_numpy(p.ops.copy()).cuda().requires_grad_(True)
    y = torch.from_numpy(_rand_like(rng, p.psi_size)).cuda().requires_grad_(True)
    x = torch.from_numpy(_rand_like(rng, p.sigma_size)).cuda()
    f = torch.dot(x, heff_apply(h, ops, y))
    f.backward()
    g_ops, g_y = ops.grad.detach().clone(), y.grad.detach().clone()
    eps = 1e-5
    with torch.no_grad():
        for _ in range(5):
            d_ops = torch.from_numpy(_rand_like(rng, p.ops.size)).cuda()
            d_y = torch.from_numpy(_rand_like(rng, p.psi_size)).cuda()
            fp = torch.dot(x, heff_apply(h, ops + eps * d_ops, y + eps * d_y)).item()
            fm = torch.dot(x, heff_apply(h, ops - eps * d_ops, y - eps * d_y)).item()
            fd = (fp - fm) / (2 * eps)
            an = (torch.dot(g_ops, d_ops) + torch.dot(g_y, d_y)).item()
            assert an == pytest.approx(fd, rel=1e-8, abs=1e-10)
    h.close()


def _sym_lowest(h, ops, v0):
    """Lowest eigenvalue of (H(ops) + H(ops)^T)/2 by ARPACK with GPU products
    (H v by b2g_heff_apply, H^T v by the adjoint's ket gradient)."""
    sla = pytest.importorskip("scipy.sparse.linalg")
    n = h.psi_size
    h.set_ops(ops)

    def mv(v):
        vd = torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64).ravel()).cuda()
        s = torch.zeros(n, dtype=torch.float64, device="cuda")
        t = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        h(vd, s)
        h.adjoint(vd, None, None, t)
        h.ctx.synchronize()
        return (0.5 * (s + t)).cpu().numpy()

    op = sla.LinearOperator((n, n), matvec=mv, dtype=np.float64)
    w = sla.eigsh(op, k=1, which="SA", v0=v0, tol=1e-14, return_eigenvectors=False)
    return float(w[0])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hub8_su2", "hub16_su2_M250"])
def test_converged_energy_gradient_matches_finite_differences(problems, ctx, name):
    """Hellmann-Feynman gradient of the lowest eigenvalue (device Davidson +
    adjoint, through torch.autograd) vs central differences of the lowest
    eigenvalue of the symmetrised H_eff(ops + t D) in 20 random directions."""
    from b2g.autodiff import converged_energy
    p = problems[name]
    h = _heff(ctx, p)
    ops = torch.from_numpy(p.ops.copy()).cuda().requires_grad_(True)
    psi0 = p.extra.get("psi_final", p.psi)
    e, v = converged_energy(h, ops, psi0, conv_thrd=1e-20)
    e.backward()
    g = ops.grad.detach().clone()
    if "davidson_energy" in p.meta:
        assert e.item() == pytest.approx(p.meta["davidson_energy"], abs=1e-8)
    v0 = v.cpu().numpy()
    rng = np.random.default_rng(9)
    scale = float(np.sqrt(np.mean(p.ops ** 2)))
    eps = 1e-5
    worst = 0.0
    for _ in range(20):
        d = torch.from_numpy(_rand_like(rng, p.ops.size, scale)).cuda()
        with torch.no_grad():
            ep = _sym_lowest(h, (ops + eps * d).contiguous(), v0)
            em = _sym_lowest(h, (ops - eps * d).contiguous(), v0)
        fd = (ep - em) / (2 * eps)
        an = torch.dot(g, d).item()
        worst = max(worst, abs(an - fd) / max(abs(fd), 1e-12))
    assert worst <= RTOL_FD_EIG, worst
    h.close()


@pytest.mark.gpu
def test_gpu_integral_gradient_matches_reference_differences(ctx):
    """The same through the product path: device Davidson (FP64) for the site
    energy, the adjoint kernel for dE/dops via torch.autograd, chained to the
    integrals; against the reference's central differences (<= 1e-6)."""
    from b2g.autodiff import chain_to_parameters, converged_energy
    from b2g.capi import PairSeq
    from b2g.problem import PAIR_FIELDS
    z, meta = _grad_fixture()
    seq = PairSeq({k: z[k] for k in PAIR_FIELDS})
    n = int(z["psi_size"])
    h = b2g.EffectiveHamiltonian(ctx, seq, z["ops"], n, int(z["sigma_size"]))
    ops = torch.from_numpy(np.array(z["ops"])).cuda().requires_grad_(True)
    e, _ = converged_energy(h, ops, z["psi"], conv_thrd=1e-20)
    e.backward()
    assert e.item() == pytest.approx(meta["energy"], abs=1e-10)
    dE = chain_to_parameters(ops.grad, z["jac_idx"], z["jac_val"], z["jac_ptr"])
    _check_integral_gradient(dE, z, meta)
    h.close()


@pytest.mark.gpu
def test_gpu_integral_gradient_matches_reference_pdm(ctx):
    """The adjoint kernel at the converged MPS centre, chained to the integrals,
    against the reference's 1-/2-PDM (<= 1e-6)."""
    from b2g.autodiff import chain_to_parameters
    from b2g.capi import PairSeq
    from b2g.problem import PAIR_FIELDS
    z, meta = _grad_fixture("syn8_su2_conv_grad")
    seq = PairSeq({k: z[k] for k in PAIR_FIELDS})
    h = b2g.EffectiveHamiltonian(ctx, seq, z["ops"], int(z["psi_size"]), int(z["sigma_size"]))
    v = torch.from_numpy(z["psi"] / np.linalg.norm(z["psi"])).cuda()
    g = torch.zeros(z["ops"].size, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    h.adjoint(v, v, g, None)
    ctx.synchronize()
    _check_pdm_derivative(chain_to_parameters(g, z["jac_idx"], z["jac_val"], z["jac_ptr"]), z, meta)
    h.close()


@pytest.mark.gpu
def test_gpu_full_integral_gradient_and_random_directions(ctx):
    """The full integral gradient from the adjoint kernel against the
    reference's 1-/2-PDM, and in 20 random directions D of integral space
    against central differences (step 1e-5) of the energy of the fixed MPS,
    <psi|H_eff(ops(theta + t D))|psi>, computed with the GPU product."""
    from b2g.autodiff import chain_to_parameters
    from b2g.capi import PairSeq
    from b2g.problem import PAIR_FIELDS
    z, meta = _grad_fixture("syn8_su2_conv_fullgrad")
    seq = PairSeq({k: z[k] for k in PAIR_FIELDS})
    n = int(z["psi_size"])
    h = b2g.EffectiveHamiltonian(ctx, seq, z["ops"], n, int(z["sigma_size"]))
    v = torch.from_numpy(z["psi"] / np.linalg.norm(z["psi"])).cuda()
    g = torch.zeros(z["ops"].size, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    h.adjoint(v, v, g, None)
    ctx.synchronize()
    dE = chain_to_parameters(g, z["jac_idx"], z["jac_val"], z["jac_ptr"])
    _check_full_gradient(dE, z["pdm_derivative"])

    def energy(ops):
        h.set_ops(np.ascontiguousarray(ops))
        s = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        h(v, s)
        ctx.synchronize()
        return float(torch.dot(v, s))

    rng = np.random.default_rng(21)
    eps, worst = 1e-5, 0.0
    for _ in range(20):
        d = rng.standard_normal(dE.size)
        jd = _jac_times(z, d)
        fd = (energy(z["ops"] + eps * jd) - energy(z["ops"] - eps * jd)) / (2 * eps)
        worst = max(worst, abs(float(dE @ d) - fd) / abs(fd))
        assert float(z["pdm_derivative"] @ d) == pytest.approx(fd, rel=1e-6)
    assert worst <= 1e-6, worst
    h.close()


@pytest.mark.gpu
def test_adjoint_argument_errors(problems, ctx):
    p = problems["hub8_su2"]
    h = _heff(ctx, p)
    x = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
    g = torch.zeros(p.ops.size, dtype=torch.float64, device="cuda")
    from b2g import capi
    # the C entry before its schedule exists: a state error, nothing launched
    rc = capi.lib().b2g_heff_adjoint(h._h, x.data_ptr(), x.data_ptr(), 1.0, g.data_ptr(), None)
    assert rc == capi.B2G_ERR_STATE
    with pytest.raises(ValueError):
        h.set_ops(np.zeros(p.ops.size + 1))
    with pytest.raises(ValueError):
        h.adjoint(x, x, torch.zeros(3, dtype=torch.float64, device="cuda"), None)
    h.close()


def test_config5_integral_gradients_record():
    """The n=16 M=500 integral-derivative run (tests/golden/make_grad_syn16.py,
    the reference's own DMRG and PDMs; its dumps are too large to keep): the
    recorded summary holds the energy identity and, in all 20 directions, the
    adjoint chain, the PDM contraction and the central differences agree to 1e-6."""
    import json
    import os

    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "syn16_M500_grad.json")) as f:
        d = json.load(f)
    assert len(d["rows"]) >= 20
    assert abs(d["energy_mps"] - d["energy_from_pdms"]) < 1e-10
    for k in ("adjoint_cpu_vs_pdm", "fd_vs_pdm", "adjoint_cpu_vs_fd"):
        assert d["max_rel_err"][k] <= d["bound"] == 1e-6, (k, d["max_rel_err"][k])
    for r in d["rows"]:
        assert abs(r["adjoint_cpu"] - r["pdm"]) <= 1e-6 * abs(r["pdm"])
