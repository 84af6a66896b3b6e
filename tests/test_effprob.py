"""Reader of the reference's EffectiveProblem export (b2g.effprob) against
files the reference wrote (EffectiveHamiltonian::save_eff_problem, through
the harness; tests/golden/make_effprob_fixtures.py) and the fields the harness
dumped from the same H_eff object in the same run: the wavefunction block
list, the connection infos with their CG factors, and the operator tensors
the H_eff expression refers to."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import GOLDEN

from b2g.effprob import read_effective_problem
from b2g.mps_io import FormatError

CASES = ("hub8_su2", "hub8_sz", "syn8_su2", "syn8_sz")


def _read(tmp_path, name):
    z = np.load(os.path.join(GOLDEN, name + "_effprob.npz"))
    p = tmp_path / (name + ".effprob")
    p.write_bytes(z["effprob"].tobytes())
    return read_effective_problem(str(p)), z


@pytest.mark.parametrize("name", CASES)
def test_header_and_wavefunction(tmp_path, name):
    d, z = _read(tmp_path, name)
    assert d["version"] == 2
    assert d["symmetry"] == ("SU2" if int(z["su2"]) else "SZ")
    assert d["isite"] == int(z["isite"]) and d["forward"] == bool(int(z["forward"]))
    for key in ("cmat", "vmat"):   # bra and ket share the block list in a ground-state solve
        m = d[key]
        info = m["info"]
        assert m["type"] == "normal"
        assert info["delta_quantum"] == int(z["dq_target"][0])
        np.testing.assert_array_equal(info["quanta"], z["wfn_q"])
        np.testing.assert_array_equal(info["n_states_bra"], z["wfn_rows"])
        np.testing.assert_array_equal(info["n_states_ket"], z["wfn_cols"])
        np.testing.assert_array_equal(info["block_shifts"], z["wfn_shift"])
        assert m["total_memory"] == int(np.sum(z["wfn_rows"].astype(np.int64) * z["wfn_cols"]))


@pytest.mark.parametrize("name", CASES)
def test_connection_infos_bit_exact(tmp_path, name):
    """The exported wavefunction connection infos (the objects b2g_wfn_connection
    restates) equal the harness's dump of the same objects, bit for bit."""
    d, z = _read(tmp_path, name)
    terms = [t for t in d["terms"] if t["cinfo"] is not None]
    assert [t["operator_quantum"] for t in terms] == [int(x) for x in z["ci_opdq"]]
    for j, t in enumerate(terms):
        ci = t["cinfo"]
        np.testing.assert_array_equal(ci["n"], z["ci_n"][5 * j:5 * j + 5])
        q0, q1 = int(z["ci_qstart"][j]), int(z["ci_qstart"][j + 1])
        np.testing.assert_array_equal(ci["quanta"], z["ci_q"][q0:q1])
        np.testing.assert_array_equal(ci["idx"], z["ci_idx"][q0:q1])
        s0, s1 = int(z["ci_start"][j]), int(z["ci_start"][j + 1])
        assert ci["nc"] == s1 - s0
        np.testing.assert_array_equal(ci["stride"], z["ci_stride"][s0:s1])
        assert np.array_equal(ci["factor"].view(np.uint64), z["ci_factor"][s0:s1].view(np.uint64))
        for k in ("ia", "ib", "ic"):
            np.testing.assert_array_equal(ci[k], z["ci_" + k][s0:s1])


@pytest.mark.parametrize("name", CASES)
def test_operator_tensors_and_expression(tmp_path, name):
    """Each exported operator's matrix carries the operator's quantum label and
    block shifts that tile its blocks; the H_eff expression (a sum of products of a
    left and a right operator, and of operators with delayed sums) refers only
    to operators the left and right tensors (or the delayed list) export."""
    d, _ = _read(tmp_path, name)
    op = d["op"]
    assert op["delayed"] and op["lopt"] is not None and op["ropt"] is not None

    def key(e):
        return (e["name"], e["site_index"], e["q_label"])

    sides = {}
    for side in ("lopt", "ropt"):
        keys = set()
        for e, m in op[side]["ops"]:
            info = m["info"]
            if e["type"] == "elem":
                assert e["q_label"] == info["delta_quantum"]
                keys.add(key(e))
            if m["type"] == "normal":
                # the blocks tile the matrix; its size is recorded as 0 when the
                # operator's data is not in memory at export time
                sizes = info["n_states_bra"].astype(np.int64) * info["n_states_ket"]
                assert m["total_memory"] in (0, int(sizes.sum()))
                np.testing.assert_array_equal(info["block_shifts"],
                                              np.concatenate([[0], np.cumsum(sizes)[:-1]]))
        sides[side] = keys
    known = sides["lopt"] | sides["ropt"] | {key(e) for e in op["dops"] if e["type"] == "elem"}
    expr = op["mat"]["data"][0]
    strings = expr["strings"] if expr["type"] == "sum" else [expr]
    assert len(strings) > 0
    for s in strings:
        assert s["type"] in ("prod", "sumprod")
        if s["type"] == "prod":
            # left operand from the left tensor, right operand from the right one
            assert s["a"] is None or key(s["a"]) in sides["lopt"]
            assert s["b"] is None or key(s["b"]) in sides["ropt"]
        else:
            # a product with a (delayed) sum: every operand is an exported operator
            for x in [s["a"], s["b"], s["c"], *s["ops"]]:
                assert x is None or x["type"] != "elem" or key(x) in known


def test_truncated_and_foreign_files_raise(tmp_path):
    z = np.load(os.path.join(GOLDEN, "hub8_su2_effprob.npz"))
    raw = z["effprob"].tobytes()
    p = tmp_path / "cut.effprob"
    p.write_bytes(raw[:len(raw) // 2])
    with pytest.raises(FormatError):
        read_effective_problem(str(p))
    p.write_bytes(b"NOTANEFF" + raw[8:])
    with pytest.raises(FormatError):
        read_effective_problem(str(p))
    p.write_bytes(raw + b"\0")
    with pytest.raises(FormatError):
        read_effective_problem(str(p))
