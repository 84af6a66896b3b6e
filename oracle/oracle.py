"""Python access to the C restatement in b2g_oracle.c -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
legs, always as the checker or the timed CPU reference, never as the product.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "libb2g_oracle.so")
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "block2-preview_gb300"))

from b2g.capi import PairSeq, PairSeqC  # noqa: E402  (the boundary's plain-data struct)

_lib = None


def build():
    src = os.path.join(HERE, "b2g_oracle.c")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["bash", os.path.join(HERE, "build.sh")], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.b2g_oracle_load_blas.argtypes = [C.c_char_p, C.c_char_p]
        L.b2g_oracle_load_blas.restype = C.c_int
        L.b2g_oracle_blas_loaded.restype = C.c_int
        L.b2g_oracle_replay.argtypes = [C.POINTER(PairSeqC), C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_uint64, C.c_double, C.c_int]
        L.b2g_oracle_replay.restype = C.c_int
        L.b2g_oracle_syev.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.b2g_oracle_davidson.argtypes = [C.POINTER(PairSeqC), C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_uint64, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L.b2g_oracle_davidson.restype = C.c_int
        _lib = L
    return _lib


def find_blas():
    """Path of scipy's bundled OpenBLAS (symbols prefixed scipy_), or None."""
    try:
        import scipy
    except ImportError:
        return None
    d = os.path.join(os.path.dirname(scipy.__file__), os.pardir, "scipy.libs")
    c = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    return os.path.abspath(c[0]) if c else None


def load_blas() -> bool:
    if lib().b2g_oracle_blas_loaded():
        return True
    p = find_blas()
    if p is None:
        return False
    return lib().b2g_oracle_load_blas(p.encode(), b"scipy_") == 0


def replay(seq: PairSeq, ops, psi, sigma_size, scale=1.0, nthreads=1, sigma=None):
    ops = np.ascontiguousarray(ops, dtype=np.float64)
    psi = np.ascontiguousarray(psi, dtype=np.float64)
    out = np.zeros(sigma_size) if sigma is None else sigma
    rc = lib().b2g_oracle_replay(C.byref(seq.c), ops.ctypes.data, psi.ctypes.data, out.ctypes.data,
                                 sigma_size, scale, nthreads)
    if rc != 0:
        raise RuntimeError("oracle replay failed")
    return out


def syev(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    m = a.shape[0]
    w = np.zeros(m)
    v = np.zeros((m, m))
    lib().b2g_oracle_syev(m, a.ctypes.data, w.ctypes.data, v.ctypes.data)
    return w, v


def davidson(seq: PairSeq, ops, diag, psi0, conv_thrd, max_iter=500, def_min=2, def_max=50, nthreads=1):
    psi = np.array(psi0, dtype=np.float64, copy=True)
    e = C.c_double()
    it = C.c_int()
    ops = np.ascontiguousarray(ops, dtype=np.float64)
    diag = np.ascontiguousarray(diag, dtype=np.float64)
    rc = lib().b2g_oracle_davidson(C.byref(seq.c), ops.ctypes.data, diag.ctypes.data, psi.ctypes.data,
                                   psi.size, conv_thrd, max_iter, def_min, def_max, nthreads,
                                   C.byref(e), C.byref(it))
    return e.value, it.value, psi, rc


def dm_truncate(trace_right, psi_dm, psi_rows, psi_cols, psi_off, dm_dim, psi, k, cutoff):
    """Density-matrix truncation restated in numpy (the checker of b2g_dm_truncate).

    rho: OperatorFunctions::trans_product without noise
    (src/core/operator_functions.hpp:777-838); selection:
    MovingEnvironment::truncate_density_matrix, Physical
    (src/dmrg/moving_environment.hpp:3715-3843); split: split_density_matrix
    (moving_environment.hpp:4250-4345) with normalize = True.
    Returns (eigenvalues per block ascending, kept per block, rotation blocks,
    wavefunction blocks per psi block, discarded weight)."""
    nb = len(dm_dim)
    rho = [np.zeros((int(n), int(n))) for n in dm_dim]
    blocks = []
    for a in range(len(psi_dm)):
        r, c, o = int(psi_rows[a]), int(psi_cols[a]), int(psi_off[a])
        P = np.asarray(psi[o:o + r * c]).reshape(r, c)
        blocks.append(P)
        b = int(psi_dm[a])
        if b >= 0:
            rho[b] += P @ P.T if trace_right else P.T @ P
    eigs, vecs = [], []
    for b in range(nb):
        w, v = np.linalg.eigh(rho[b]) if dm_dim[b] else (np.zeros(0), np.zeros((0, 0)))
        eigs.append(w)
        vecs.append(v)           # columns = eigenvectors, ascending
    ss = [(b, j) for b in range(nb) for j in range(int(dm_dim[b]))]
    k_total, error = len(ss), 0.0
    if k != -1:
        ss.sort(key=lambda p: -eigs[p[0]][p[1]])
        for i in range(k, k_total):
            x = eigs[ss[i][0]][ss[i][1]]
            if x > 0:
                error += x
        kk = min(k, k_total)
        while kk > 1 and eigs[ss[kk - 1][0]][ss[kk - 1][1]] < cutoff:
            x = eigs[ss[kk - 1][0]][ss[kk - 1][1]]
            if x > 0:
                error += x
            kk -= 1
        ss = sorted(ss[:kk])
    kept = np.zeros(nb, dtype=np.int32)
    sel = [[] for _ in range(nb)]
    for b, j in ss:
        kept[b] += 1
        sel[b].append(j)
    rots = []
    for b in range(nb):
        if kept[b] == 0:
            rots.append(None)
            continue
        V = vecs[b][:, sel[b]]                     # dm_dim x kept
        rots.append(V.copy() if trace_right else V.T.copy())
    wfns = []
    for a in range(len(psi_dm)):
        b = int(psi_dm[a])
        if b < 0 or kept[b] == 0:
            wfns.append(None)
        elif trace_right:
            wfns.append(rots[b].T @ blocks[a])
        else:
            wfns.append(blocks[a] @ rots[b].T)
    nrm = np.sqrt(sum(float((x * x).sum()) for x in wfns if x is not None))
    wfns = [None if x is None else x / nrm for x in wfns]
    return eigs, kept, rots, wfns, error


def block_contract(rec, env, site, tmp_size, out_size):
    """Environment blocking replayed from block-level records (the checker of
    b2g_block_contract): iadd records (OperatorFunctions::iadd,
    src/core/operator_functions.hpp:135-170) then Kronecker records
    (GMatrixFunctions::tensor_product, src/core/matrix_functions.hpp:1269-1400),
    in recorded order."""
    tmp = np.zeros(int(tmp_size))
    out = np.zeros(int(out_size))
    blobs = [np.asarray(env, dtype=np.float64), np.asarray(site, dtype=np.float64), tmp]
    for q in range(len(rec["ia_m"])):
        m, n = int(rec["ia_m"][q]), int(rec["ia_n"][q])
        src = blobs[int(rec["ia_src_blob"][q])]
        so, do = int(rec["ia_src"][q]), int(rec["ia_dst"][q])
        if rec["ia_conj"][q]:
            b = src[so:so + m * n].reshape(n, m).T
        else:
            b = src[so:so + m * n].reshape(m, n)
        tmp[do:do + m * n] += float(rec["ia_f"][q]) * b.ravel()
    for q in range(len(rec["kr_am"])):
        am, an, bm, bn = (int(rec[k][q]) for k in ("kr_am", "kr_an", "kr_bm", "kr_bn"))
        A = blobs[int(rec["kr_ablob"][q])][int(rec["kr_a"][q]):][:am * an].reshape(am, an)
        B = blobs[int(rec["kr_bblob"][q])][int(rec["kr_b"][q]):][:bm * bn].reshape(bm, bn)
        if rec["kr_ca"][q]:
            A = A.T
        if rec["kr_cb"][q]:
            B = B.T
        K = float(rec["kr_f"][q]) * np.kron(A, B)
        cn, c = int(rec["kr_cn"][q]), int(rec["kr_c"][q])
        rows, cols = K.shape
        for r in range(rows):
            out[c + r * cn:c + r * cn + cols] += K[r]
    return out


def _view_idx(off, rows, cols, ld):
    return int(off) + np.arange(rows)[:, None] * int(ld) + np.arange(cols)[None, :]


def adjoint(seq: PairSeq, ops, x, y):
    """Gradients of f = <x| H_eff(ops) |y> in numpy (the checker of b2g_heff_adjoint).

    H_eff(ops) y is the replay above: per pair, W = alpha0 y[a0:] op_b0(ops[b0:])
    and sigma[c1:] += alpha1 op_a1(ops[a1:]) W (BatchGEMMSeq::rotate,
    src/core/batch_gemm.hpp:893-902).  Differentiating f pair by pair gives
    df/dA' = c x_p (y_p B')^T, df/dB' = c y_p^T (A'^T x_p), df/dy_p = c A'^T x_p B'^T
    with c = alpha0 alpha1, A' = op_a1(A), B' = op_b0(B).  Returns (grad_ops, grad_y)."""
    a = seq.arrays
    ops = np.asarray(ops, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    gops = np.zeros_like(ops)
    gy = np.zeros_like(y)
    for p in range(seq.n):
        m0, n0, k0 = int(a["m0"][p]), int(a["n0"][p]), int(a["k0"][p])
        m1, n1, k1 = int(a["m1"][p]), int(a["n1"][p]), int(a["k1"][p])
        c = float(a["alpha0"][p]) * float(a["alpha1"][p])
        iy = _view_idx(a["a0"][p], m0, k0, a["lda0"][p])
        ix = _view_idx(a["c1"][p], m1, n1, a["ldc1"][p])
        tb, ta = int(a["tb0"][p]), int(a["ta1"][p])
        ib = _view_idx(a["b0"][p], n0, k0, a["ldb0"][p]) if tb else _view_idx(a["b0"][p], k0, n0, a["ldb0"][p])
        ia = _view_idx(a["a1"][p], k1, m1, a["lda1"][p]) if ta else _view_idx(a["a1"][p], m1, k1, a["lda1"][p])
        Bp = ops[ib].T if tb else ops[ib]
        Ap = ops[ia].T if ta else ops[ia]
        yp, xp = y[iy], x[ix]
        W = yp @ Bp
        T = Ap.T @ xp
        dA = c * (xp @ W.T)
        dB = c * (yp.T @ T)
        np.add.at(gops, ia, dA.T if ta else dA)
        np.add.at(gops, ib, dB.T if tb else dB)
        np.add.at(gy, iy, c * (T @ Bp.T))
    return gops, gy
