"""Autotuner of the tensor-core tile shapes (b2g_heff_autotune): every
candidate it times is a valid plan, the kept plan is installed, and H_eff*psi
through it still matches the reference (TF32x3 tolerance; FP64 exact)."""
import numpy as np
import pytest

from conftest import fixture_ids

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import b2g  # noqa: E402

RTOL_TF32X3 = 2e-5   # split-TF32 x3 on tensor cores, FP32 accumulation
RTOL_FP64 = 1e-12


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = b2g.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", fixture_ids())
def test_autotune_keeps_a_correct_plan(problems, ctx, name):
    p = problems[name]
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    try:
        psi = torch.from_numpy(p.psi).cuda()
        sig = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        h(psi, sig, 1.0, b2g.TF32X3)       # images and a graph-cache entry before re-planning
        h(psi, sig, 1.0, b2g.TF32X3)
        ctx.synchronize()
        r = h.autotune()
        assert 1 <= len(r["candidates"]) <= 12 and 0 <= r["best"] < len(r["candidates"])
        assert all(c["ms"] > 0 for c in r["candidates"])
        kept = r["candidates"][r["best"]]
        assert h.params == {k: kept[k] for k in ("g0_tile_cols", "g1_tile_cols", "g1_chunk")}
        assert h.graph_count == 0
        for form, tol in ((b2g.TF32X3, RTOL_TF32X3), (b2g.FP64, RTOL_FP64)):
            for _ in range(3):   # direct, captured, replayed
                sig.zero_()
                torch.cuda.synchronize()
                h(psi, sig, 1.0, form)
                ctx.synchronize()
                h.status()
                assert rel(sig.cpu().numpy(), p.sigma) <= tol
    finally:
        h.close()


def test_autotune_rejects_other_forms_and_sequences(problems, ctx):
    p = problems["hub8_su2"]
    q = problems["hub8_sz"]
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    try:
        with pytest.raises(b2g.B2GError):
            h.autotune(form=b2g.FP64)
        h.seq = q.seq()
        with pytest.raises(b2g.B2GError):
            h.autotune()
    finally:
        h.close()


def test_set_params_installs_given_shapes(problems, ctx):
    p = problems["hub16_su2_M250"]
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    try:
        psi = torch.from_numpy(p.psi).cuda()
        for shapes in ((128, 128, 16), (256, 128, 64), (256, 256, 32)):
            h.set_params(*shapes)
            assert h.params == dict(zip(("g0_tile_cols", "g1_tile_cols", "g1_chunk"), shapes))
            sig = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            h(psi, sig, 1.0, b2g.TF32X3)
            ctx.synchronize()
            h.status()
            assert rel(sig.cpu().numpy(), p.sigma) <= RTOL_TF32X3
        with pytest.raises(b2g.B2GError):
            h.set_params(64, 256, 32)
        with pytest.raises(b2g.B2GError):
            h.set_params(256, 256, 65)
    finally:
        h.close()
