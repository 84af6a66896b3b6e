"""The H_eff's wavefunction connection info (ConnectionInfo::initialize_wfn,
src/core/sparse_matrix.hpp:163-292) restated by b2g_wfn_connection, against
the reference's own connection infos dumped by the harness (tests/golden/
*_cinfo.npz): the index arrays (conj-type boundaries, sub-label starts, bra /
left-op / right-op / ket block indices, in the reference's order) bit for
bit, the Clebsch-Gordan factors (SU(2) 9j x transposition x fermion sign)
to 1e-14."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from b2g import quanta

CINFO = sorted(glob.glob(os.path.join(GOLDEN, "*_cinfo.npz")))


def test_cinfo_fixtures_exist():
    names = {os.path.basename(p) for p in CINFO}
    assert {"hub8_su2_cinfo.npz", "hub8_sz_cinfo.npz", "syn8_su2_cinfo.npz", "syn8_sz_cinfo.npz"} <= names


@pytest.mark.parametrize("path", CINFO, ids=[os.path.basename(p)[:-4] for p in CINFO])
def test_wfn_connection_matches_reference(path):
    z = np.load(path)
    sym = quanta.SU2 if int(z["su2"]) else quanta.SZ
    cdq, vdq = (int(x) for x in z["cdq_vdq"])
    qs, st = z["ci_qstart"], z["ci_start"]
    left = (z["lop_dq"], z["lop_ferm"], z["lop_start"], z["lop_q"])
    right = (z["rop_dq"], z["rop_ferm"], z["rop_start"], z["rop_q"])
    assert z["ci_opdq"].size >= 1
    for i in range(z["ci_opdq"].size):
        n = z["ci_n"][5 * i:5 * i + 5]
        q = z["ci_q"][qs[i]:qs[i + 1]]
        # the sub-labels (inputs) with their conj types, read off the reference's boundaries
        conj = np.array([next(t for t in range(4) if n[t] <= k < n[t + 1]) for k in range(q.size)])
        r = quanta.wfn_connection(sym, cdq, vdq, int(z["ci_opdq"][i]), conj, q, left, right,
                                  z["wfn_q"], z["bra_q"])
        a, b = st[i], st[i + 1]
        assert np.array_equal(r["n"], n)
        assert np.array_equal(r["idx"], z["ci_idx"][qs[i]:qs[i + 1]])
        for k in ("stride", "ia", "ib", "ic"):
            assert np.array_equal(r[k], z["ci_" + k][a:b]), k
        assert np.allclose(r["factor"], z["ci_factor"][a:b], rtol=1e-14, atol=1e-14)
        if sym == quanta.SZ:
            assert np.all(np.abs(r["factor"]) == 1.0)


def test_recoupling_identities():
    """Spot checks of the SU(2) recoupling algebra through the SU(2) connection
    info of a trivial case: a spin-0 operator pair acting on a singlet block
    gives factor 1."""
    s0 = quanta.su2_label(0, 0)
    left = (np.array([s0], np.uint64), np.array([0]), np.array([0, 1]), np.array([s0], np.uint64))
    right = left
    r = quanta.wfn_connection(quanta.SU2, s0, s0, s0, np.array([0]), np.array([s0], np.uint64), left, right,
                              np.array([s0], np.uint64), np.array([s0], np.uint64))
    assert r["stride"].size == 1 and r["factor"][0] == pytest.approx(1.0, abs=1e-15)


def test_wfn_connection_rejects_bad_input():
    s0 = quanta.su2_label(0, 0)
    ops = (np.array([s0], np.uint64), np.array([0]), np.array([0, 1]), np.array([s0], np.uint64))
    q = np.array([s0], np.uint64)
    with pytest.raises(Exception):
        quanta.wfn_connection(7, s0, s0, s0, np.array([0]), q, ops, ops, q, q)   # unknown symmetry
    with pytest.raises(Exception):
        quanta.wfn_connection(quanta.SU2, s0, s0, s0, np.array([5]), q, ops, ops, q, q)   # conj type 5
    # a sub-label whose operator delta quantum has no operator info
    s2 = quanta.su2_label(0, 2)
    with pytest.raises(Exception):
        quanta.wfn_connection(quanta.SU2, s0, s0, s2, np.array([0]), np.array([s2], np.uint64), ops, ops, q, q)
