"""The drop-in's H_eff dump format (b2g_block2::HeffDump in
block2-preview_gb300/shim/b2g_block2.hpp: one raw little-endian array per
field plus manifest.txt with "name dtype count" lines and "#key value"
scalars) read back by b2g.problem.load_dump, on a golden problem written in
that format: the loaded pairs, blob and vectors equal the source, and the
oracle's replay of the loaded problem reproduces the reference's sigma."""
import os

import numpy as np

from conftest import GOLDEN

from b2g.capi import PAIR_F64_FIELDS, PAIR_INT_FIELDS, PAIR_U64_FIELDS
from b2g.problem import load_dump, load_problem
from oracle import oracle


def _write_dump(d, prob):
    d.mkdir()
    lines = []

    def arr(name, a, dt):
        np.ascontiguousarray(a, dtype={"i4": "<i4", "u8": "<u8", "f8": "<f8"}[dt]).tofile(str(d / (name + ".bin")))
        lines.append(f"{name} {dt} {np.asarray(a).size}")
    for k in PAIR_INT_FIELDS:
        arr(k, prob.pairs[k], "i4")
    for k in PAIR_F64_FIELDS:
        arr(k, prob.pairs[k], "f8")
    for k in PAIR_U64_FIELDS:
        arr(k, prob.pairs[k], "u8")
    arr("ops", prob.ops, "f8")
    arr("psi", prob.psi, "f8")
    arr("diag", prob.diag, "f8")
    arr("psi_converged", prob.psi[::-1], "f8")
    lines += [f"#psi_size {prob.psi_size}", f"#sigma_size {prob.sigma_size}", "#isweep 1", "#site 3",
              "#conv_thrd 1e-10", "#const_e 0.5"]
    (d / "manifest.txt").write_text("\n".join(lines) + "\n")


def test_dump_round_trip(tmp_path):
    prob = load_problem(os.path.join(GOLDEN, "hub8_su2.npz"))
    _write_dump(tmp_path / "dump", prob)
    got = load_dump(str(tmp_path / "dump"))
    assert got.psi_size == prob.psi_size and got.sigma_size == prob.sigma_size
    for k in PAIR_INT_FIELDS + PAIR_F64_FIELDS + PAIR_U64_FIELDS:
        np.testing.assert_array_equal(got.pairs[k], prob.pairs[k])
    np.testing.assert_array_equal(got.ops, prob.ops)
    np.testing.assert_array_equal(got.psi, prob.psi)
    np.testing.assert_array_equal(got.diag, prob.diag)
    np.testing.assert_array_equal(got.extra["psi_converged"], prob.psi[::-1])
    assert got.meta["site"] == 3 and got.meta["const_e"] == 0.5
    sig = oracle.replay(got.seq(), got.ops, got.psi, got.sigma_size)
    assert np.linalg.norm(sig - prob.sigma) <= 1e-12 * np.linalg.norm(prob.sigma)
