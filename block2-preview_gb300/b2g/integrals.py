"""Hamiltonian integrals for the benchmark problems: seeded synthetic ab initio
integrals and the 1D Hubbard chain, plus a FCIDUMP writer/reader.

Synthetic ab initio recipe (n orbitals, restricted spin, no point group):

* h_pp ~ U[-2, 2], sorted ascending;
* h_pq = h_qp ~ N(0, sigma = 0.05 * exp(-|p-q|/4)) for p != q;
* (pq|rs) = sum_{L<3n} B^L_pq B^L_rs with B^L_pq = B^L_qp ~ N(0, sigma = 0.3 * exp(-|p-q|/4)),
  which is positive semidefinite and has the 8-fold permutational symmetry.

Generator (fixed, so every consumer sees identical integrals for a seed):
``numpy.random.default_rng(seed)``; draws in this order:
1. ``uniform(-2, 2, n)``  -> h_pp (then sorted);
2. ``standard_normal(n*(n-1)//2)`` -> h_pq for p > q, row-major over (p, q<p);
3. ``standard_normal((3n, n*(n+1)//2))`` -> B^L_pq for p >= q, row-major over (p, q<=p).

The FCIDUMP layout is the Molpro one that the reference reads
(src/core/integral.hpp:745 ``FCIDUMP::read``): unique (ij|kl) with i>=j, k>=l,
ij>=kl, then h_ij with i>=j, then the core energy, 1-based indices.
"""
from __future__ import annotations

import numpy as np


def synthetic_integrals(n: int, seed: int = 0):
    """Return (h1e[n,n], eri[n,n,n,n], ecore) for the synthetic recipe."""
    rng = np.random.default_rng(seed)
    hd = np.sort(rng.uniform(-2.0, 2.0, n))
    p_idx, q_idx = np.tril_indices(n, -1)
    off = rng.standard_normal(p_idx.size) * 0.05 * np.exp(-np.abs(p_idx - q_idx) / 4.0)
    h = np.zeros((n, n))
    h[np.arange(n), np.arange(n)] = hd
    h[p_idx, q_idx] = off
    h[q_idx, p_idx] = off
    nl = 3 * n
    pl, ql = np.tril_indices(n, 0)
    z = rng.standard_normal((nl, pl.size)) * 0.3 * np.exp(-np.abs(pl - ql) / 4.0)[None, :]
    b = np.zeros((nl, n, n))
    b[:, pl, ql] = z
    b[:, ql, pl] = z
    bm = b.reshape(nl, n * n)
    eri = (bm.T @ bm).reshape(n, n, n, n)
    return h, eri, 0.0


def hubbard_integrals(n: int, t: float = 1.0, u: float = 4.0):
    """1D open-boundary Hubbard chain in the reference's convention
    (src/core/hubbard.hpp:31-80): h_{i,i+1} = t, (ii|ii) = U."""
    h = np.zeros((n, n))
    for i in range(n - 1):
        h[i, i + 1] = h[i + 1, i] = t
    eri = np.zeros((n, n, n, n))
    for i in range(n):
        eri[i, i, i, i] = u
    return h, eri, 0.0


def write_fcidump(path: str, h, eri, ecore: float, nelec: int, ms2: int = 0, tol: float = 0.0):
    n = h.shape[0]
    lines = [
        f" &FCI NORB={n:4d},NELEC={nelec:4d},MS2={ms2:4d},",
        "  ORBSYM=" + ",".join(["1"] * n) + ",",
        "  ISYM=1,",
        " &END",
    ]
    pairs = [(i, j) for i in range(n) for j in range(i + 1)]
    out = []
    for a, (i, j) in enumerate(pairs):
        for (k, l) in pairs[: a + 1]:
            v = eri[i, j, k, l]
            if abs(v) > tol:
                out.append(f"{v: .16e} {i + 1:4d} {j + 1:4d} {k + 1:4d} {l + 1:4d}")
    for (i, j) in pairs:
        v = h[i, j]
        if abs(v) > tol:
            out.append(f"{v: .16e} {i + 1:4d} {j + 1:4d}    0    0")
    out.append(f"{ecore: .16e}    0    0    0    0")
    with open(path, "w") as f:
        f.write("\n".join(lines + out) + "\n")


def read_fcidump(path: str):
    """Return (h1e, eri, ecore, norb, nelec, ms2) from a FCIDUMP file (8-fold symmetric)."""
    with open(path) as f:
        text = f.read()
    head, body = text.split("&END", 1) if "&END" in text else text.split("/", 1)
    hdr = head.replace("&FCI", "").replace("\n", " ")
    import re

    def grab(key, default=0):
        m = re.search(key + r"\s*=\s*(-?\d+)", hdr, re.I)
        return int(m.group(1)) if m else default

    n, nelec, ms2 = grab("NORB"), grab("NELEC"), grab("MS2")
    h = np.zeros((n, n))
    eri = np.zeros((n, n, n, n))
    ecore = 0.0
    for ln in body.strip().splitlines():
        t = ln.split()
        if len(t) != 5:
            continue
        v = float(t[0])
        i, j, k, l = (int(x) - 1 for x in t[1:])
        if i < 0:
            ecore = v
        elif k < 0:
            h[i, j] = h[j, i] = v
        else:
            for (a, b, c, d) in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k)):
                eri[a, b, c, d] = eri[c, d, a, b] = v
    return h, eri, ecore, n, nelec, ms2
