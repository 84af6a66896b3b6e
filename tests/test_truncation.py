"""Density-matrix truncation (the step after Davidson in the two-site sweep).

The golden fixtures *_dm.npz hold the reference's own density matrix, its
per-block spectrum, the discarded weight and the split tensors for the
converged wavefunction of each fixture site (MovingEnvironment::
density_matrix + split_density_matrix, src/dmrg/moving_environment.hpp:
3554-3580, 4250-4345).  The oracle restatement is pinned to them on the CPU;
the GPU path (b2g_dm_truncate) is checked against both.

Eigenvectors are fixed only up to sign (and rotation inside a degenerate
eigenvalue group), so the split is compared through products that do not
depend on that choice: rotation * wavefunction, blockwise, which is the
truncated wavefunction itself.
"""
from __future__ import annotations

import glob
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402

DM_FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*_dm.npz")))
DM_IDS = [os.path.basename(p)[:-len("_dm.npz")] for p in DM_FIXTURES]


def load(path):
    z = np.load(path)
    d = {k: z[k] for k in z.files}
    d["meta"] = json.loads(str(d["meta"]))
    d["trace_right"] = bool(d["trace_right"])
    return d


def ref_blocks(d, tag):
    out = []
    for r, c, o in zip(d[tag + "_rows"], d[tag + "_cols"], d[tag + "_off"]):
        out.append(d[tag + "_data"][int(o):int(o) + int(r) * int(c)].reshape(int(r), int(c)))
    return out


def ref_split(d):
    """Reference split as (kept per dm block, {psi block: truncated psi block})."""
    tr = d["trace_right"]
    left, right = ref_blocks(d, "left"), ref_blocks(d, "right")
    rot_side, wfn_side = ("left", "right") if tr else ("right", "left")
    rot = {int(b): m for b, m in zip(d[rot_side + "_link"], left if tr else right)}
    wfn = {int(a): m for a, m in zip(d[wfn_side + "_link"], right if tr else left)}
    kept = np.zeros(d["dm_dim"].size, dtype=np.int32)
    for b, m in rot.items():
        kept[b] = m.shape[1] if tr else m.shape[0]
    recon = {}
    for a, w in wfn.items():
        b = int(d["psi_dm"][a])
        recon[a] = rot[b] @ w if tr else w @ rot[b]
    return kept, recon


def recon_of(layout_psi_dm, trace_right, rots, wfns):
    out = {}
    for a, w in enumerate(wfns):
        if w is None:
            continue
        b = int(layout_psi_dm[a])
        out[a] = rots[b] @ w if trace_right else w @ rots[b]
    return out


def eig_blocks(d):
    out, pos = [], 0
    for n in d["dm_dim"]:
        out.append(d["dm_eig"][pos:pos + int(n)])
        pos += int(n)
    return out


def oracle_split(d, k=None, cutoff=None):
    return oracle.dm_truncate(d["trace_right"], d["psi_dm"], d["psi_rows"], d["psi_cols"],
                              d["psi_off"], d["dm_dim"], d["psi"],
                              int(d["bond_dim"]) if k is None else k,
                              float(d["cutoff"]) if cutoff is None else cutoff)


def compare_recon(ours, ref, tol):
    assert set(ours) == set(ref)
    for a in ref:
        np.testing.assert_allclose(ours[a], ref[a], atol=tol, rtol=0)


EIG_NOISE = 1e-13   # absolute accuracy of a dense symmetric eigensolver on |rho| ~ 1


def recon_tol(d, eig_ref):
    """Tolerance of the truncated wavefunction.  Eigenvalues closer than the
    solver noise to the cut (ties, or a cut among the numerically-zero
    eigenvalues) leave the kept subspace undetermined inside that cluster; the
    truncated wavefunction then differs by at most sqrt(cluster weight).
    With a clean gap at the cut it is 1e-10."""
    k = int(d["bond_dim"])
    w = np.sort(np.concatenate(eig_ref))[::-1]
    if k <= 0 or k >= w.size:
        return 1e-10
    cut = w[k - 1]
    cluster = np.abs(w - cut) < EIG_NOISE
    if abs(w[k - 1] - w[k]) >= EIG_NOISE:
        return 1e-10
    return 1e-10 + 2 * np.sqrt(cluster.sum() * (abs(cut) + EIG_NOISE))


@pytest.mark.skipif(not DM_FIXTURES, reason="no *_dm.npz fixtures")
@pytest.mark.parametrize("path", DM_FIXTURES, ids=DM_IDS)
def test_oracle_matches_reference_truncation(path):
    d = load(path)
    full = d["meta"].get("split_tensors", True)   # the large case keeps spectrum + weight only
    # density matrix blocks, in the reference's block layout
    nb = d["dm_dim"].size
    rho = [np.zeros((int(n), int(n))) for n in d["dm_dim"]]
    for a in range(d["psi_dm"].size):
        r, c, o = int(d["psi_rows"][a]), int(d["psi_cols"][a]), int(d["psi_off"][a])
        P = d["psi"][o:o + r * c].reshape(r, c)
        if d["psi_dm"][a] >= 0:
            rho[d["psi_dm"][a]] += P @ P.T if d["trace_right"] else P.T @ P
    for b in range(nb):
        n, o = int(d["dm_dim"][b]), int(d["dm_off"][b])
        if full:
            np.testing.assert_allclose(rho[b], d["rho"][o:o + n * n].reshape(n, n), atol=1e-13, rtol=0)
    eigs, kept, rots, wfns, err = oracle_split(d)
    eig_ref = eig_blocks(d)
    for b in range(nb):
        np.testing.assert_allclose(eigs[b], eig_ref[b], atol=1e-13, rtol=0)
    assert err == pytest.approx(float(d["error"]), abs=1e-13, rel=1e-9)
    if not full:
        return
    kept_ref, recon_ref = ref_split(d)
    tol = recon_tol(d, eig_ref)
    if tol == 1e-10:
        np.testing.assert_array_equal(kept, kept_ref)
    compare_recon(recon_of(d["psi_dm"], d["trace_right"], rots, wfns), recon_ref, tol)


@pytest.mark.skipif(not DM_FIXTURES, reason="no *_dm.npz fixtures")
def test_fixture_truncation_is_nontrivial():
    """At least one fixture actually discards states (error > 0) and at least
    one traces out each side."""
    ds = [load(p) for p in DM_FIXTURES]
    assert any(float(d["error"]) > 0 for d in ds)
    assert {d["trace_right"] for d in ds} == {True, False}


# ---------------------------------------------------------------- GPU path
def gpu_split(ctx, d, k=None, cutoff=None):
    from b2g.truncation import DensityMatrixLayout, split_density_matrix
    lay = DensityMatrixLayout(d["trace_right"], d["psi_dm"], d["psi_rows"], d["psi_cols"],
                              d["psi_off"], d["dm_dim"])
    return split_density_matrix(ctx, lay, d["psi"], int(d["bond_dim"]) if k is None else k,
                                float(d["cutoff"]) if cutoff is None else cutoff)


@pytest.fixture(scope="module")
def ctx():
    from b2g.heff import Context
    c = Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", DM_FIXTURES, ids=DM_IDS)
def test_gpu_truncation_matches_reference(ctx, path):
    d = load(path)
    res = gpu_split(ctx, d)
    eig_ref = eig_blocks(d)
    for b in range(d["dm_dim"].size):
        np.testing.assert_allclose(res.eigenvalues[b], eig_ref[b], atol=1e-13, rtol=0)
    assert res.error == pytest.approx(float(d["error"]), abs=1e-13, rel=1e-9)
    if not d["meta"].get("split_tensors", True):
        # large case: the split is checked against the oracle instead
        eigs, kept, rots, wfns, err = oracle_split(d)
        tol = recon_tol(d, eig_ref)
        if tol == 1e-10:
            np.testing.assert_array_equal(res.kept, kept)
        compare_recon(recon_of(d["psi_dm"], d["trace_right"], res.rotation, res.wavefunction),
                      recon_of(d["psi_dm"], d["trace_right"], rots, wfns), tol)
        return
    kept_ref, recon_ref = ref_split(d)
    tol = recon_tol(d, eig_ref)
    if tol == 1e-10:
        np.testing.assert_array_equal(res.kept, kept_ref)
    compare_recon(recon_of(d["psi_dm"], d["trace_right"], res.rotation, res.wavefunction),
                  recon_ref, tol)
    # the rotation blocks are orthonormal (the new MPS tensor is left/right canonical)
    for b, R in enumerate(res.rotation):
        if R is None:
            continue
        G = R.T @ R if d["trace_right"] else R @ R.T
        np.testing.assert_allclose(G, np.eye(G.shape[0]), atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("k", [-1, 1, 7, 10 ** 6])
def test_gpu_truncation_bond_dims_vs_oracle(ctx, k):
    """k = -1 keeps everything, k = 1 keeps one state, k above the total keeps
    all -- each against the oracle on a fixture wavefunction.  The cutoff is
    below every eigenvalue, so the numerically-zero ones (whose signs are
    solver noise) are not dropped by it."""
    d = load(DM_FIXTURES[0])
    res = gpu_split(ctx, d, k=k, cutoff=-1.0)
    eigs, kept, rots, wfns, err = oracle_split(d, k=k, cutoff=-1.0)
    assert res.error == pytest.approx(err, abs=1e-13)
    np.testing.assert_array_equal(res.kept, kept)
    ours = recon_of(d["psi_dm"], d["trace_right"], res.rotation, res.wavefunction)
    compare_recon(ours, recon_of(d["psi_dm"], d["trace_right"], rots, wfns), 1e-10)


def random_layout(rng, nb, maxdim, trace_right, with_orphan=True):
    dims = rng.integers(0, maxdim + 1, size=nb).astype(np.int32)
    dims[0] = maxdim                      # one full-size block
    rows, cols, dm, off, pos = [], [], [], [], 0
    for b in range(nb):
        if dims[b] == 0:
            continue
        for _ in range(int(rng.integers(1, 4))):
            other = int(rng.integers(1, maxdim + 1))
            r, c = (dims[b], other) if trace_right else (other, dims[b])
            rows.append(r), cols.append(c), dm.append(b), off.append(pos)
            pos += r * c
    if with_orphan:                       # a psi block that maps to no dm block
        rows.append(3), cols.append(2), dm.append(-1), off.append(pos)
        pos += 6
    return dict(trace_right=trace_right, psi_dm=np.array(dm, np.int32),
                psi_rows=np.array(rows, np.int32), psi_cols=np.array(cols, np.int32),
                psi_off=np.array(off, np.uint64), dm_dim=dims), pos


@pytest.mark.gpu
@pytest.mark.parametrize("trace_right", [True, False])
@pytest.mark.parametrize("maxdim", [1, 33, 300])
def test_gpu_truncation_random_blocks(ctx, trace_right, maxdim):
    """Ragged random layouts (empty dm blocks, a psi block outside every dm
    block, a 300-state block) against the oracle; the spectrum sums to |psi|^2
    and the kept + discarded weight is the whole."""
    from b2g.truncation import DensityMatrixLayout, split_density_matrix
    rng = np.random.default_rng(1000 + maxdim + int(trace_right))
    lay, n = random_layout(rng, 9, maxdim, trace_right)
    psi = rng.standard_normal(n)
    psi /= np.linalg.norm(psi)
    k = max(1, int(lay["dm_dim"].sum()) // 3)
    res = split_density_matrix(ctx, DensityMatrixLayout(**lay), psi, k, 1e-14)
    eigs, kept, rots, wfns, err = oracle.dm_truncate(lay["trace_right"], lay["psi_dm"], lay["psi_rows"],
                                                     lay["psi_cols"], lay["psi_off"], lay["dm_dim"],
                                                     psi, k, 1e-14)
    for b in range(lay["dm_dim"].size):
        np.testing.assert_allclose(res.eigenvalues[b], eigs[b], atol=1e-13, rtol=0)
    np.testing.assert_array_equal(res.kept, kept)
    assert res.error == pytest.approx(err, abs=1e-13)
    compare_recon(recon_of(lay["psi_dm"], trace_right, res.rotation, res.wavefunction),
                  recon_of(lay["psi_dm"], trace_right, rots, wfns), 1e-10)
    orphan = psi[int(lay["psi_off"][-1]):int(lay["psi_off"][-1]) + 6]
    total = sum(float(e.sum()) for e in res.eigenvalues)
    assert total == pytest.approx(1.0 - float(orphan @ orphan), abs=1e-12)
    kept_w = sum(float(np.sort(e)[::-1][:int(m)].sum()) for e, m in zip(res.eigenvalues, res.kept))
    assert kept_w + res.error == pytest.approx(total, abs=1e-12)


@pytest.mark.gpu
def test_gpu_truncation_rejects_bad_layout(ctx):
    from b2g.capi import B2GError
    from b2g.truncation import DensityMatrixLayout, split_density_matrix
    lay = DensityMatrixLayout(True, np.array([0], np.int32), np.array([4], np.int32),
                              np.array([2], np.int32), np.array([0], np.uint64),
                              np.array([3], np.int32))          # rows 4 != dm size 3
    with pytest.raises(B2GError):
        split_density_matrix(ctx, lay, np.ones(8), 2)
    lay = DensityMatrixLayout(True, np.array([5], np.int32), np.array([3], np.int32),
                              np.array([2], np.int32), np.array([0], np.uint64),
                              np.array([3], np.int32))          # dm block 5 does not exist
    with pytest.raises(B2GError):
        split_density_matrix(ctx, lay, np.ones(6), 2)
