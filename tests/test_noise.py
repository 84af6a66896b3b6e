"""Perturbative noise (EffectiveHamiltonian::perturbative_noise,
src/dmrg/effective_hamiltonian.hpp:262-433) on the H_eff engine.

The fixtures hold the single GEMMs block2 records for that product in Tasked
mode, the operator blob they read, the converged ket and the reference's
perturbed-wavefunction group (tests/golden/make_noise_fixtures.py; forward
sweeps apply op(L) to the ket, backward sweeps op(R)).  b2g_noise_pairs turns
the GEMM list into H_eff pairs (an identity block on the side a GEMM lacks);
the oracle's replay of those pairs and the GPU product must give the
reference's group."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, noise_ids
import b2g
from b2g import capi
from b2g.noise import GEMM_F64, GEMM_I32, GEMM_U64, GemmList, PerturbativeNoise, noise_pairs, with_identity
from oracle import oracle

FIELDS = GEMM_I32 + GEMM_F64 + GEMM_U64


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files if k != "meta"}
    d["meta"] = json.loads(str(z["meta"]))
    d["gemms"] = GemmList({k: d["g_" + ("akind" if k == "a_kind" else "bkind" if k == "b_kind" else k)]
                           for k in FIELDS})
    return d


def pairs_of(d, gemms=None):
    return noise_pairs(gemms or d["gemms"], d["psi"].size, d["ops"].size, d["sigma"].size,
                       d["blk_off"], d["blk_rows"], d["blk_cols"])


def test_fixtures_cover_both_directions_and_symmetries():
    metas = [load(n)["meta"] for n in noise_ids()]
    assert len(metas) >= 6
    assert {m["forward"] for m in metas} == {0, 1}
    assert any(m["n_ket_left"] > 0 for m in metas) and any(m["n_ket_right"] > 0 for m in metas)
    assert any("_sz" in m["name"] for m in metas) and any("_su2" in m["name"] for m in metas)
    # ReducedPerturbative, Perturbative (one vector per perturbation) and the LowMem variant
    assert {m["noise_type"] for m in metas} == {12, 4, 76}


@pytest.mark.parametrize("name", noise_ids())
def test_group_layout_tiles_sigma(name):
    d = load(name)
    sizes = d["blk_rows"].astype(np.int64) * d["blk_cols"]
    np.testing.assert_array_equal(d["blk_off"], np.concatenate([[0], np.cumsum(sizes)[:-1]]))
    assert int(sizes.sum()) == d["sigma"].size
    assert np.all(np.diff(d["blk_vec"]) >= 0) and d["blk_vec"].max() + 1 == d["meta"]["n_vectors"]


@pytest.mark.parametrize("name", noise_ids())
def test_oracle_replay_of_noise_pairs_matches_reference(name):
    """The pairs b2g_noise_pairs makes, replayed by the oracle (the reference's
    Tasked pair replay restated), give the reference's perturbed group."""
    d = load(name)
    seq, dim = pairs_of(d)
    m = d["meta"]
    assert seq.n == int(np.count_nonzero((d["g_m"] > 0) & (d["g_n"] > 0) & (d["g_k"] > 0) & (d["g_alpha"] != 0)))
    a = seq.arrays
    on_left, on_right = a["a1"] == d["ops"].size, a["b0"] == d["ops"].size  # pairs reading the identity
    assert np.all(on_left | on_right) and not np.any(on_left & on_right)
    assert dim == max(int(a["m1"][on_left].max(initial=0)), int(a["n0"][on_right].max(initial=0)))
    assert np.all(a["lda1"][on_left] == dim) and np.all(a["ldb0"][on_right] == dim)
    ops = with_identity(d["ops"], dim)
    out = oracle.replay(seq, ops, d["psi"], d["sigma"].size, nthreads=2)
    assert rel(out, d["sigma"]) <= 1e-13, m["name"]
    st = b2g.plan_stats(seq, ops.size, d["psi"].size, d["sigma"].size)
    assert st["n_pairs"] == seq.n and st["n_regions"] >= 1


def _one(d, **change):
    a = {k: np.array(v, copy=True) for k, v in d["gemms"].arrays.items()}
    for k, v in change.items():
        a[k][0] = v
    return GemmList(a)


def test_noise_pairs_rejects_bad_lists():
    d = load("hub8_su2_noise")
    psi_n, sig_n = d["psi"].size, d["sigma"].size
    g = d["gemms"].arrays
    ket_is_b = int(g["b_kind"][0]) == 0
    for change, code in (({"beta": 0.0}, capi.B2G_ERR_ARG),
                         ({"a_kind": int(g["b_kind"][0])}, capi.B2G_ERR_ARG),
                         ({"c": sig_n}, capi.B2G_ERR_ARG),
                         ({"c": np.uint64(2**64 - 1)}, capi.B2G_ERR_ARG),
                         ({("b" if ket_is_b else "a"): psi_n}, capi.B2G_ERR_ARG),
                         ({("a" if ket_is_b else "b"): np.uint64(2**64 - 8)}, capi.B2G_ERR_ARG)):
        with pytest.raises(b2g.B2GError) as e:
            pairs_of(d, _one(d, **change))
        assert e.value.code == code, change
    # a transposed ket operand that is not one contiguous row
    k = "tb" if ket_is_b else "ta"
    rows = int(g["k"][0]) if ket_is_b else int(g["m"][0])
    if rows > 1:
        with pytest.raises(b2g.B2GError) as e:
            pairs_of(d, _one(d, **{k: 1}))
        assert e.value.code in (capi.B2G_ERR_UNSUPPORTED, capi.B2G_ERR_ARG)


def test_noise_pairs_of_an_empty_list():
    """A site whose noise product records nothing (block2 skips a site without
    the identity operator on one side) gives no pairs."""
    gl = GemmList({k: [] for k in FIELDS})
    seq, dim = noise_pairs(gl, 4, 0, 4, [0], [2], [2])
    assert seq.n == 0 and dim == 0


def test_per_row_form_is_transposed_as_a_whole():
    """AdvancedGEMM::multiply's per-row form (src/core/batch_gemm.hpp:584-607):
    c[r, :] (as an m x 1 column, ld 1) += alpha op(A)^T (m x k) * ket[r, :]^T
    becomes one pair with the ket row on the left; checked against numpy."""
    rng = np.random.default_rng(5)
    k, m, rows = 6, 4, 3
    ket = rng.standard_normal(rows * k)          # rows x k, row-major
    op = rng.standard_normal(k * m)              # k x m operator block, row-major
    group = np.zeros(rows * m)                   # rows x m output block
    gl = GemmList({"ta": [1] * rows, "tb": [1] * rows, "m": [m] * rows, "n": [1] * rows, "k": [k] * rows,
                   "lda": [m] * rows, "ldb": [k] * rows, "ldc": [1] * rows, "a_kind": [1] * rows,
                   "b_kind": [0] * rows, "alpha": [0.5] * rows, "beta": [1.0] * rows,
                   "a": [0] * rows, "b": [r * k for r in range(rows)], "c": [r * m for r in range(rows)]})
    seq, dim = noise_pairs(gl, ket.size, op.size, group.size, [0], [rows], [m])
    assert seq.n == rows and dim == 1
    assert np.all(seq.arrays["m0"] == 1) and np.all(seq.arrays["ldc1"] == m)
    out = oracle.replay(seq, with_identity(op, dim), ket, group.size)
    want = 0.5 * ket.reshape(rows, k) @ op.reshape(k, m)
    np.testing.assert_allclose(out.reshape(rows, m), want, rtol=1e-14, atol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("name", noise_ids())
def test_gpu_noise_matches_reference(name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    d = load(name)
    ctx = b2g.Context(0)
    nz = PerturbativeNoise(ctx, d["gemms"], d["ops"], d["psi"].size, d["sigma"].size,
                           d["blk_off"], d["blk_rows"], d["blk_cols"])
    x = torch.from_numpy(d["psi"]).cuda()
    for form, tol in ((b2g.FP64, 1e-12), (b2g.TF32X3, 2e-5)):
        y = torch.zeros(d["sigma"].size, dtype=torch.float64, device="cuda")
        nz(x, y, form)
        nz.status()
        assert rel(y.cpu().numpy(), d["sigma"]) <= tol, form
    nz.close()
    ctx.close()
