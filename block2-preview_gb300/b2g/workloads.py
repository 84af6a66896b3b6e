"""Named H_eff workloads for benchmarking.

Each workload is one two-site effective Hamiltonian at the middle site of a
DMRG sweep, as recorded by the reference (its GEMM-pair sequence).  Small
ones carry the reference's own operator values (tests/golden); large ones
(workloads/*.npz) carry the reference's recorded structure only, factored
(tables of distinct psi sub-blocks, right/left operator blocks and sigma
sub-blocks plus four table indices per pair), with seeded synthetic operator
values of the recorded blob size: the throughput of H_eff*psi depends on the
structure, not on the values.
"""
from __future__ import annotations

import json
import os

import numpy as np

from .problem import HeffProblem, load_problem

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_ROOT = os.path.dirname(_PKG)
GOLDEN = os.path.join(_ROOT, "tests", "golden")
STRUCTS = os.path.join(_PKG, "workloads")

WORKLOADS = {
    "heff_hub16_su2_M250": ("golden", os.path.join(GOLDEN, "hub16_su2_M250.npz")),
    "heff_syn8_su2_M60": ("golden", os.path.join(GOLDEN, "syn8_su2.npz")),
    "heff_syn8_sz_M50": ("golden", os.path.join(GOLDEN, "syn8_sz.npz")),
    "heff_syn24_su2_M1000_sweep0": ("struct", os.path.join(STRUCTS, "heff_syn24_su2_M1000_sweep0.npz")),
    "heff_syn24_su2_M1000_mid": ("struct", os.path.join(STRUCTS, "heff_syn24_su2_M1000_mid.npz")),
}
DEFAULT = "heff_syn24_su2_M1000_mid"


def pack(a: dict, s: dict, description: str) -> dict:
    """Factored form of a recorded pair sequence (arrays a, scalars s of a dump)."""
    def tab(keys):
        arr = np.stack([a[k].astype(np.int64) for k in keys], 1)
        u, inv = np.unique(arr, axis=0, return_inverse=True)
        return u, inv.ravel().astype(np.int32)

    pt, pi = tab(["a0", "m0", "k0", "lda0"])
    rt, ri = tab(["b0", "tb0", "k0", "n0", "ldb0"])
    lt, li = tab(["a1", "ta1", "m1", "k1", "lda1"])
    st, si = tab(["c1", "m1", "n1", "ldc1"])
    a0u, a0i = np.unique(a["alpha0"], return_inverse=True)
    a1u, a1i = np.unique(a["alpha1"], return_inverse=True)
    if a0u.size >= 65536 or a1u.size >= 65536:
        raise ValueError("too many distinct coefficients for 16-bit indices")
    meta = {k: s[k] for k in ("n_pairs", "psi_size", "sigma_size", "ops_size", "mnk", "isweep", "site",
                              "n_sites")}
    meta["description"] = description
    return dict(pt=pt, rt=rt, lt=lt, st=st, idx=np.stack([pi, ri, li, si], 1),
                a0u=a0u, a0i=a0i.ravel().astype(np.uint16), a1u=a1u, a1i=a1i.ravel().astype(np.uint16),
                psi_block_rows=a["psi_block_rows"], psi_block_cols=a["psi_block_cols"],
                psi_block_shift=a["psi_block_shift"],
                meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8))


def unpack(z) -> tuple[dict, dict]:
    """Inverse of pack: the b2g_pair_seq arrays and the metadata."""
    idx = z["idx"]
    p, r, l, s = z["pt"][idx[:, 0]], z["rt"][idx[:, 1]], z["lt"][idx[:, 2]], z["st"][idx[:, 3]]
    pairs = {
        "a0": p[:, 0], "m0": p[:, 1], "k0": p[:, 2], "lda0": p[:, 3],
        "b0": r[:, 0], "tb0": r[:, 1], "n0": r[:, 3], "ldb0": r[:, 4],
        "a1": l[:, 0], "ta1": l[:, 1], "m1": l[:, 2], "k1": l[:, 3], "lda1": l[:, 4],
        "c1": s[:, 0], "n1": s[:, 2], "ldc1": s[:, 3],
        "alpha0": z["a0u"][z["a0i"]], "alpha1": z["a1u"][z["a1i"]],
    }
    return pairs, json.loads(bytes(z["meta"]).decode())


def synthetic_problem(path: str, seed: int = 0) -> HeffProblem:
    """Recorded structure + seeded synthetic operator values and psi."""
    z = np.load(path)
    pairs, meta = unpack(z)
    rng = np.random.default_rng(seed)
    n_ops = int(meta["ops_size"])
    # random sign and mantissa, exponent fixed: values uniform in +-[0.0625, 0.125);
    # a 2^24-value random pool (not a multiple of any block size) repeated over the blob
    pool = np.frombuffer(rng.bytes(8 * ((1 << 24) + 7)), dtype=np.uint64).copy()
    pool &= np.uint64(0x800FFFFFFFFFFFFF)
    pool |= np.uint64(0x3FB0000000000000)
    ops = np.resize(pool.view(np.float64), n_ops)
    psi = rng.standard_normal(int(meta["psi_size"]))
    psi /= np.linalg.norm(psi)
    meta = dict(meta, data="reference-recorded structure; seeded synthetic operator values "
                           "(random sign, |x| uniform in [1/16,1/8)) and psi (normal, normalized)")
    return HeffProblem(pairs=pairs, ops=ops, psi_size=int(meta["psi_size"]),
                       sigma_size=int(meta["sigma_size"]), psi=psi, meta=meta)


def get(name: str) -> HeffProblem:
    if name not in WORKLOADS:
        raise KeyError(f"unknown workload {name!r}; known: {sorted(WORKLOADS)}")
    kind, path = WORKLOADS[name]
    if kind == "struct":
        return synthetic_problem(path)
    p = load_problem(path)
    p.meta.setdefault("data", "reference operator values (golden fixture)")
    return p
