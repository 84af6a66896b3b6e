"""PDM expectations (block2's fast expectation algorithm,
TensorFunctions::tensor_product_expectation, src/core/tensor_functions.hpp:1701-1877)
as GEMM pairs of the H_eff engine (b2g.npdm).

Each fixture is one site of the reference's 1-PDM or 2-PDM Expect sweep on a
converged MPS (tests/golden/make_npdm_fixtures.py): the partial <bra| a |ket>
of every unique left operator recorded as pairs, the reference's partials,
the dot terms and the reference's expectation values.  Here the oracle (the
reference's Tasked pair replay restated) runs the pairs; the partials and the
expectation values built from them must equal the reference's."""
import os

import numpy as np
import pytest

from conftest import ROOT, npdm_ids
import b2g
from b2g.npdm import expectations, normal_layout
from npdm_fixture import load
from oracle import oracle


def test_fixtures_cover_orders_symmetries_and_transposed_partials():
    metas = [load(n)["meta"] for n in npdm_ids()]
    assert len(metas) >= 5
    assert {m["order"] for m in metas} == {1, 2}
    assert any("_sz" in m["name"] for m in metas) and any("_su2" in m["name"] for m in metas)
    assert all(int(np.sum(load(n)["p_trans"])) > 0 for n in npdm_ids())


@pytest.mark.parametrize("name", npdm_ids())
def test_partials_and_expectations_match_reference(name):
    d = load(name)
    L, T = d["layout"], d["terms"]
    out = oracle.replay(d["seq"], d["ops"], d["psi"], d["sigma"].size, nthreads=2)
    scale = max(np.linalg.norm(d["sigma"]), 1e-300)
    assert np.linalg.norm(out - d["sigma"]) / scale <= 1e-13
    e = expectations(normal_layout(out, L["p_trans"], L["p_nblk"], L["b_off"], L["b_rows"], L["b_cols"]),
                     L["p_off"], d["meta"]["n_expect"], T["t_k"], T["t_part"], T["t_roff"], T["t_rsize"],
                     T["t_f"], d["rmats"])
    ref = d["expect"]
    assert np.abs(e - ref).max() <= 1e-13 * max(np.abs(ref).max(), 1.0)
    st = b2g.plan_stats(d["seq"], d["ops"].size, d["psi"].size, d["sigma"].size)
    assert st["n_pairs"] == d["seq"].n


def test_partial_blocks_tile_the_partials():
    for name in npdm_ids():
        d = load(name)
        L = d["layout"]
        size = L["b_rows"].astype(np.int64) * L["b_cols"]
        np.testing.assert_array_equal(L["b_off"], np.concatenate([[0], np.cumsum(size)[:-1]]))
        assert int(size.sum()) == d["sigma"].size
        assert int(L["p_nblk"].sum()) == L["b_off"].size


REF_BIN = os.path.join(ROOT, "oracle", "_ref", "dmrg_sweep_ref")
# Hubbard L=8 U=4 at half filling, M=40: the 1-PDM after the sweeps (block2's Expect)
HUB8_PDM = dict(ham="hubbard", L=8, U=4.0, t=1.0, sym="su2", M=(40,), sweeps=4, noises=(1e-4, 1e-5, 0.0, 0.0),
                dav=(1e-10,), seed=1234, pdm=1)


@pytest.mark.skipif(not os.path.exists(REF_BIN), reason="block2 reference build absent")
def test_reference_sweep_reports_the_1pdm(tmp_path):
    from b2g.sweep import run_sweep
    r = run_sweep(binary=REF_BIN, arms=("cpu",), threads=2, workdir=str(tmp_path), **HUB8_PDM)
    p = np.array(r["arms"][0]["pdm1"]).reshape(8, 8)
    assert abs(np.trace(p) - 8.0) < 1e-10 and np.abs(p - p.T).max() < 1e-12
