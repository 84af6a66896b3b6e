"""The reference's on-disk MPS format (b2g.mps_io): files written by the
reference itself (tests/golden/mps_*: the final MPS of a Hubbard L=8 run,
SU(2) and SZ, copied from the harness's scratch directory) are read and
written back byte for byte, and the right-canonical site tensors read this
way have orthonormal rows per bra label (the reference's gauge)."""
import glob
import os
from collections import defaultdict

import numpy as np
import pytest

from conftest import GOLDEN
from b2g import mps_io, quanta

CASES = {"mps_hub8_su2": quanta.SU2, "mps_hub8_sz": quanta.SZ}


@pytest.mark.parametrize("case", sorted(CASES))
def test_every_file_round_trips_byte_for_byte(case):
    d = os.path.join(GOLDEN, case)
    files = sorted(glob.glob(os.path.join(d, "F.MPS.*")))
    assert len(files) >= 10
    for f in files:
        raw = open(f, "rb").read()
        name = os.path.basename(f)
        if name.endswith(".-1"):
            obj = mps_io.parse_header(raw)
        elif ".INFO." in name:
            obj = mps_io.parse_state_info(raw)
        else:
            obj = mps_io.parse_site_tensor(raw)
        assert obj.to_bytes() == raw, name


@pytest.mark.parametrize("case", sorted(CASES))
def test_load_save_mps(case, tmp_path):
    d = os.path.join(GOLDEN, case)
    m = mps_io.load_mps(d)
    assert m.header.n_sites == 8 and m.header.dot == 2
    assert len(m.left_dims) == len(m.right_dims) == m.header.n_sites + 1
    assert all(t is not None for t in m.tensors)
    mps_io.save_mps(str(tmp_path), m)
    for f in glob.glob(os.path.join(d, "F.MPS.*")):
        assert open(f, "rb").read() == open(os.path.join(tmp_path, os.path.basename(f)), "rb").read()


@pytest.mark.parametrize("case", sorted(CASES))
def test_right_canonical_tensors_are_orthonormal(case):
    sym = CASES[case]
    m = mps_io.load_mps(os.path.join(GOLDEN, case))
    checked = 0
    for i, t in enumerate(m.tensors):
        if m.header.canonical_form[i] != "R":
            continue
        rows = defaultdict(list)
        for b in range(t.quanta.size):
            rows[quanta.op(sym, quanta.BRA, int(t.quanta[b]), t.delta_quantum)].append(t.block(b))
        for blks in rows.values():
            M = np.hstack(blks)
            assert np.abs(M @ M.T - np.eye(M.shape[0])).max() <= 1e-13
        checked += 1
    assert checked >= 6


def test_truncated_files_are_rejected():
    f = sorted(glob.glob(os.path.join(GOLDEN, "mps_hub8_su2", "F.MPS.KET.3")))[0]
    raw = open(f, "rb").read()
    with pytest.raises(mps_io.FormatError):
        mps_io.parse_site_tensor(raw[:-8])
    with pytest.raises(mps_io.FormatError):
        mps_io.parse_header(b"\x08\x00\x00\x00" * 3 + b"CR")
