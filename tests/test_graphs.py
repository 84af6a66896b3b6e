"""CUDA-graph replay of repeated H_eff*psi applies: a replayed apply gives the
bit-identical sigma of the direct launches (same kernels, fixed order), keeps
the c += scale * H b semantics, survives buffer growth, stays bounded, and
leaves Davidson unchanged."""
import numpy as np
import pytest

from conftest import fixture_ids

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import b2g  # noqa: E402


@pytest.fixture(scope="module")
def ctx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = b2g.Context(0)
    yield c
    c.close()


def run(h, ctx, psi, sig, scale, form, init=0.0):
    sig.fill_(init)
    torch.cuda.synchronize()
    h(psi, sig, scale, form)
    ctx.synchronize()
    h.status()
    return sig.cpu().numpy().copy()


@pytest.mark.parametrize("name", fixture_ids())
@pytest.mark.parametrize("form", [b2g.FP64, b2g.TF32X3])
def test_replay_is_bit_identical(problems, ctx, name, form):
    p = problems[name]
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    try:
        psi = torch.from_numpy(p.psi).cuda()
        sig = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
        h.set_graphs(False)
        ref = run(h, ctx, psi, sig, 0.75, form, init=0.5)
        h.set_graphs(True)
        outs = [run(h, ctx, psi, sig, 0.75, form, init=0.5) for _ in range(4)]
        assert h.graph_count == 1
        for o in outs:
            assert np.array_equal(o, ref)
        if form == b2g.FP64:
            want = 0.5 + 0.75 * p.sigma
            assert np.linalg.norm(ref - want) <= 1e-12 * np.linalg.norm(want)
    finally:
        h.close()


def test_graphs_dropped_on_root_growth_and_bounded(problems, ctx):
    p = problems["hub8_su2"]
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    try:
        psi = torch.from_numpy(p.psi).cuda()
        sig = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
        ref = run(h, ctx, psi, sig, 1.0, b2g.FP64)
        run(h, ctx, psi, sig, 1.0, b2g.FP64)
        assert h.graph_count == 1
        # two roots reallocate the per-root buffers: every graph is dropped
        xb = torch.stack([psi, 2.0 * psi])
        yb = torch.zeros((2, p.sigma_size), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        h.apply_batch(xb, yb)
        ctx.synchronize()
        assert h.graph_count == 0
        assert np.array_equal(yb[0].cpu().numpy(), ref)
        # replays after the growth use the new buffers
        for _ in range(3):
            assert np.array_equal(run(h, ctx, psi, sig, 1.0, b2g.FP64), ref)
        # many argument sets: the cache stays bounded (LRU)
        many = torch.zeros((70, p.sigma_size), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for _ in range(2):
            for i in range(70):
                h(psi, many[i])
        ctx.synchronize()
        assert h.graph_count <= 64
        got = many.cpu().numpy()
        assert np.array_equal(got[0], 2.0 * ref)   # 0 + s + s: doubling is exact
        for i in range(70):
            assert np.array_equal(got[i], got[0])
    finally:
        h.close()


@pytest.mark.parametrize("form", [b2g.FP64, b2g.TF32X3])
def test_davidson_same_with_and_without_graphs(problems, ctx, form):
    p = problems["hub16_su2_M250"]
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    try:
        res = []
        for on in (False, True):
            h.set_graphs(on)
            psi = p.psi.copy()
            e, it, _, _ = h.eigs(p.diag, psi, conv_thrd=1e-10, form=form)
            res.append((e, it, psi))
        assert res[0][0] == res[1][0] and res[0][1] == res[1][1]
        assert np.array_equal(res[0][2], res[1][2])
    finally:
        h.close()
