"""Quantum-number bookkeeping (host only, no GPU) against the reference's own
values at each fixture site (tests/golden/*_qn.npz, dumped by the reference
harness where MovingEnvironment::contract_two_dot builds the two-site
wavefunction, src/dmrg/moving_environment.hpp:3376-3387): the tensor
products, the connection info and the wavefunction's block list must match
bit for bit."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

from b2g import quanta as Q  # noqa: E402

QN = sorted(glob.glob(os.path.join(GOLDEN, "*_qn.npz")))
IDS = [os.path.basename(p)[:-len("_qn.npz")] for p in QN]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + "_qn.npz"))
    si = {k[:-2]: (z[k], z[k[:-2] + "_n"].astype(np.uint32)) for k in z.files
          if k.endswith("_q") and k[:-2] + "_n" in z.files}
    return z, si


def test_fixtures_present():
    assert len(QN) >= 5


@pytest.mark.parametrize("name", IDS)
def test_tensor_products_match_reference(name):
    z, si = load(name)
    sym = Q.SU2 if int(z["su2"]) else Q.SZ
    ll = Q.tensor_product(sym, si["l"], si["ml"], cref=si["lfci"])
    rr = Q.tensor_product(sym, si["mr"], si["r"], cref=si["rfci"])
    for got, want in ((ll, si["ll"]), (rr, si["rr"])):
        assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    target = int(z["dq_target"][1])
    lt = Q.tensor_product(sym, si["l"], si["ml"], target=target)
    assert np.array_equal(lt[0], si["lt"][0]) and np.array_equal(lt[1], si["lt"][1])


@pytest.mark.parametrize("name", IDS)
def test_connection_info_matches_reference(name):
    z, si = load(name)
    sym = Q.SU2 if int(z["su2"]) else Q.SZ
    acc, ij = Q.connection_info(sym, si["l"], si["ml"], si["ll"])
    assert np.array_equal(acc, z["lc_acc"].astype(np.uint32))
    assert np.array_equal(ij[:, 0], z["lc_i"].astype(np.uint32))
    assert np.array_equal(ij[:, 1], z["lc_j"].astype(np.uint32))


@pytest.mark.parametrize("name", IDS)
def test_wavefunction_blocks_match_reference(name):
    z, si = load(name)
    sym = Q.SU2 if int(z["su2"]) else Q.SZ
    dq = int(z["dq_target"][0])
    q, rows, cols, shifts, total = Q.wavefunction_blocks(sym, si["ll"], si["rr"], dq, wfn=bool(z["is_wfn"]))
    assert np.array_equal(q, z["wfn_q"])
    assert np.array_equal(rows, z["wfn_rows"].astype(np.uint32))
    assert np.array_equal(cols, z["wfn_cols"].astype(np.uint32))
    assert np.array_equal(shifts.astype(np.uint64), z["wfn_shift"])
    assert total == int(z["total_memory"])


def test_label_arithmetic():
    a = Q.su2_label(3, 1)            # N=3, S=1/2
    b = Q.su2_label(1, 1)            # N=1, S=1/2
    s = Q.op(Q.SU2, Q.ADD, a, b)     # N=4, S in {0, 1}
    assert s == Q.su2_label(4, 2, twos_low=0)
    assert Q.op(Q.SU2, Q.COUNT, s) == 2
    assert Q.op(Q.SU2, Q.ELEM, s, 0) == Q.su2_label(4, 0)
    assert Q.op(Q.SU2, Q.ELEM, s, 1) == Q.su2_label(4, 2)
    assert Q.op(Q.SU2, Q.NEG, Q.op(Q.SU2, Q.NEG, a)) == a
    assert Q.op(Q.SU2, Q.KET, s) == Q.su2_label(4, 2)
    assert Q.op(Q.SZ, Q.ADD, Q.sz_label(2, 1), Q.sz_label(1, -1)) == Q.sz_label(3, 0)
    assert Q.op(Q.SZ, Q.NEG, Q.sz_label(2, 1, 3)) == Q.sz_label(-2, -1, 3)
    assert Q.op(Q.SZ, Q.COUNT, Q.sz_label(2, 1)) == 1
    # combine: a delta quantum that cannot connect bra and ket gives the invalid label
    dq = Q.sz_label(0, 0)
    assert Q.op(Q.SZ, Q.COMBINE, dq, Q.sz_label(2, 0), Q.sz_label(2, 0)) == Q.sz_label(2, 0)
    assert Q.op(Q.SZ, Q.COMBINE, dq, Q.sz_label(2, 0), Q.sz_label(1, 1)) == 2**64 - 1


def test_bad_arguments():
    from b2g import B2GError
    with pytest.raises(B2GError):
        Q.op(7, Q.ADD, 0, 0)
    with pytest.raises(B2GError):
        Q.op(Q.SZ, 99, 0, 0)
    with pytest.raises(ValueError):
        Q.tensor_product(Q.SZ, ([0], [1]), ([0], [1]))
