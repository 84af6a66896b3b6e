"""Quantum-number bookkeeping of block2's two-site wavefunction (host only).

Mirrors the reference's label types and StateInfo / SparseMatrixInfo
operations (src/core/symmetry.hpp SZLongLong / SU2LongLong,
src/core/state_info.hpp StateInfo::tensor_product / get_connection_info,
src/core/sparse_matrix.hpp SparseMatrixInfo::initialize /
initialize_block_shifts) through the C ABI (b2g_quanta_op,
b2g_state_tensor_product, b2g_state_connection, b2g_wfn_blocks); results are
the reference's bit for bit.  A StateInfo is a pair (quanta uint64[n],
n_states uint32[n]) with ascending packed labels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .capi import check, lib

SZ, SU2 = 0, 1
ADD, NEG, COUNT, ELEM, KET, BRA, COMBINE = range(7)
UBOND_MAX = 65535   # the reference's default 16-bit ubond_t


class StateInfoC(C.Structure):
    _fields_ = [("n", C.c_int32), ("quanta", C.c_void_p), ("n_states", C.c_void_p)]


def _si(q, n):
    q = np.ascontiguousarray(q, dtype=np.uint64)
    n = np.ascontiguousarray(n, dtype=np.uint32)
    if q.shape != n.shape or q.ndim != 1:
        raise ValueError("quanta and n_states must be 1-D arrays of equal length")
    s = StateInfoC(q.size, q.ctypes.data, n.ctypes.data)
    return s, (q, n)


def su2_label(n: int, twos: int, pg: int = 0, twos_low: int | None = None) -> int:
    """SU2LongLong(n, twos_low, twos, pg) as a packed word."""
    tl = twos if twos_low is None else twos_low
    return ((n & 0xFFFF) << 48) | ((tl & 0xFFFF) << 32) | ((twos & 0xFFFF) << 16) | (pg & 0xFFFF)


def sz_label(n: int, twos: int, pg: int = 0) -> int:
    """SZLongLong(n, twos, pg) as a packed word."""
    return ((n & 0xFFFF) << 48) | ((twos & 0xFFFF) << 16) | (pg & 0xFFFF)


def op(sym: int, code: int, a: int, b: int = 0, c: int = 0) -> int:
    out = C.c_uint64()
    check(lib().b2g_quanta_op(sym, code, C.c_uint64(a), C.c_uint64(b), C.c_uint64(c), C.byref(out)))
    return out.value


def tensor_product(sym, a, b, cref=None, target=None, ubond_max=UBOND_MAX):
    """StateInfo::tensor_product(a, b, cref) or (a, b, target); a, b, cref are
    (quanta, n_states) pairs.  Returns (quanta, n_states)."""
    if (cref is None) == (target is None):
        raise ValueError("give exactly one of cref and target")
    sa, ka = _si(*a)
    sb, kb = _si(*b)
    cap = (len(cref[0]) if cref is not None else 0) + 64 * max(1, len(ka[0]) * len(kb[0]))
    qo = np.zeros(cap, dtype=np.uint64)
    no = np.zeros(cap, dtype=np.uint32)
    so = StateInfoC(cap, qo.ctypes.data, no.ctypes.data)
    if cref is not None:
        sc, kc = _si(*cref)
        check(lib().b2g_state_tensor_product(sym, ubond_max, C.byref(sa), C.byref(sb), C.byref(sc),
                                             C.c_uint64(0), C.byref(so)))
    else:
        check(lib().b2g_state_tensor_product(sym, ubond_max, C.byref(sa), C.byref(sb), None,
                                             C.c_uint64(target), C.byref(so)))
    return qo[:so.n].copy(), no[:so.n].copy()


def connection_info(sym, a, b, c):
    """StateInfo::get_connection_info(a, b, c): (acc_n_states uint32[nc + 1],
    ij uint32[npairs, 2])."""
    sa, ka = _si(*a)
    sb, kb = _si(*b)
    sc, kc = _si(*c)
    cap = 64 * max(1, len(ka[0]) * len(kb[0]))
    acc = np.zeros(len(kc[0]) + 1, dtype=np.uint32)
    ij = np.zeros(2 * cap, dtype=np.uint32)
    npairs = C.c_int64()
    check(lib().b2g_state_connection(sym, C.byref(sa), C.byref(sb), C.byref(sc), acc.ctypes.data,
                                     ij.ctypes.data, cap, C.byref(npairs)))
    return acc, ij[:2 * npairs.value].reshape(-1, 2).copy()


def wavefunction_blocks(sym, bra, ket, dq, wfn=True, align=1):
    """SparseMatrixInfo::initialize(bra, ket, dq, _, wfn) + block shifts:
    (quanta uint64, rows uint32, cols uint32, shifts uint32, total_memory)."""
    sb, kb = _si(*bra)
    sk, kk = _si(*ket)
    cap = 64 * max(1, len(kk[0]))
    q = np.zeros(cap, dtype=np.uint64)
    r = np.zeros(cap, dtype=np.uint32)
    c = np.zeros(cap, dtype=np.uint32)
    sh = np.zeros(cap, dtype=np.uint32)
    nb = C.c_int()
    tot = C.c_uint32()
    check(lib().b2g_wfn_blocks(sym, C.byref(sb), C.byref(sk), C.c_uint64(dq), int(bool(wfn)), align,
                               q.ctypes.data, r.ctypes.data, c.ctypes.data, sh.ctypes.data, cap,
                               C.byref(nb), C.byref(tot)))
    n = nb.value
    return q[:n].copy(), r[:n].copy(), c[:n].copy(), sh[:n].copy(), tot.value


class OpInfosC(C.Structure):
    _fields_ = [("n", C.c_int32), ("dq", C.c_void_p), ("fermion", C.c_void_p), ("start", C.c_void_p),
                ("quanta", C.c_void_p)]


def _ops(dq, fermion, start, q):
    arrs = (np.ascontiguousarray(dq, dtype=np.uint64), np.ascontiguousarray(fermion, dtype=np.int32),
            np.ascontiguousarray(start, dtype=np.int32), np.ascontiguousarray(q, dtype=np.uint64))
    if arrs[2].size != arrs[0].size + 1 or arrs[1].size != arrs[0].size:
        raise ValueError("operator infos: start must have n + 1 entries and fermion n")
    return OpInfosC(arrs[0].size, *(a.ctypes.data for a in arrs)), arrs


def wfn_connection(sym, cdq, vdq, opdq, sub_conj, sub_q, left, right, ket_q, bra_q):
    """ConnectionInfo::initialize_wfn (sparse_matrix.hpp:163-292) through
    b2g_wfn_connection.  left / right: (dq, fermion, start, quanta) arrays of
    the operator infos.  Returns a dict n (5), idx, stride, factor, ia, ib, ic."""
    sc = np.ascontiguousarray(sub_conj, dtype=np.int32)
    sq = np.ascontiguousarray(sub_q, dtype=np.uint64)
    kq = np.ascontiguousarray(ket_q, dtype=np.uint64)
    bq = np.ascontiguousarray(bra_q, dtype=np.uint64)
    lo, keep_l = _ops(*left)
    ro, keep_r = _ops(*right)
    n5 = np.zeros(5, dtype=np.int32)
    idx = np.zeros(max(1, sc.size), dtype=np.uint32)
    nc = C.c_int64()
    cap = 0
    while True:
        stride = np.zeros(max(1, cap), dtype=np.uint64)
        factor = np.zeros(max(1, cap))
        ia, ib, ic = (np.zeros(max(1, cap), dtype=np.uint32) for _ in range(3))
        rc = lib().b2g_wfn_connection(sym, C.c_uint64(cdq), C.c_uint64(vdq), C.c_uint64(opdq), sc.size,
                                      sc.ctypes.data, sq.ctypes.data, C.byref(lo), C.byref(ro), kq.size,
                                      kq.ctypes.data, bq.size, bq.ctypes.data, n5.ctypes.data,
                                      idx.ctypes.data, stride.ctypes.data, factor.ctypes.data,
                                      ia.ctypes.data, ib.ctypes.data, ic.ctypes.data, cap, C.byref(nc))
        if rc != 0 and nc.value > cap:
            cap = nc.value
            continue
        check(rc)
        m = nc.value
        return {"n": n5, "idx": idx[:sc.size], "stride": stride[:m], "factor": factor[:m],
                "ia": ia[:m], "ib": ib[:m], "ic": ic[:m]}
