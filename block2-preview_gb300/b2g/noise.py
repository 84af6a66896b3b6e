"""Perturbative noise on the H_eff engine.

block2's EffectiveHamiltonian::perturbative_noise
(src/dmrg/effective_hamiltonian.hpp:262-433) applies one half of H_eff to the
converged ket; in Tasked mode it is a list of single GEMMs
``group[c] += alpha op_a(A) op_b(B)`` (one operand a ket block, the other an
operator block).  ``noise_pairs`` rewrites that list as the GEMM pairs of
H_eff*psi (b2g_noise_pairs, an identity block on the side a GEMM lacks) and
``PerturbativeNoise`` runs them through the same device plan and kernels as
H_eff*psi, with the ket as psi and the perturbed-wavefunction group as sigma.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .capi import (FP64, PAIR_F64_FIELDS, PAIR_INT_FIELDS, PAIR_U64_FIELDS, GemmListC, PairArraysC,
                   PairSeq, check, lib)

NOISE_KET = 0
NOISE_OP = 1
GEMM_I32 = ("ta", "tb", "m", "n", "k", "lda", "ldb", "ldc", "a_kind", "b_kind")
GEMM_F64 = ("alpha", "beta")
GEMM_U64 = ("a", "b", "c")


class GemmList:
    """Owns the arrays of a noise GEMM list (field names of b2g_gemm_list)."""

    def __init__(self, arrays):
        n = len(arrays["m"])
        self.arrays = {}
        for keys, dt in ((GEMM_I32, np.int32), (GEMM_F64, np.float64), (GEMM_U64, np.uint64)):
            for k in keys:
                v = np.ascontiguousarray(arrays[k], dtype=dt)
                if v.shape != (n,):
                    raise ValueError(f"GEMM field {k} has shape {v.shape}, expected ({n},)")
                self.arrays[k] = v
        self.n = n
        g = GemmListC()
        g.n_gemms = n
        for k, v in self.arrays.items():
            setattr(g, k, v.ctypes.data_as(C.POINTER(np.ctypeslib.as_ctypes_type(v.dtype))))
        self.c = g


def noise_pairs(gemms: GemmList, ket_size: int, ops_size: int, group_size: int, blk_off, blk_rows, blk_cols):
    """The pair sequence of a noise GEMM list and the size of the identity
    block it reads at offset ``ops_size`` of the operator blob."""
    n = gemms.n
    out = {k: np.zeros(n, dtype=np.int32) for k in PAIR_INT_FIELDS}
    out.update({k: np.zeros(n, dtype=np.float64) for k in PAIR_F64_FIELDS})
    out.update({k: np.zeros(n, dtype=np.uint64) for k in PAIR_U64_FIELDS})
    pa = PairArraysC()
    for k, v in out.items():
        setattr(pa, k, v.ctypes.data_as(C.POINTER(np.ctypeslib.as_ctypes_type(v.dtype))))
    off = np.ascontiguousarray(blk_off, dtype=np.uint64)
    rows = np.ascontiguousarray(blk_rows, dtype=np.int32)
    cols = np.ascontiguousarray(blk_cols, dtype=np.int32)
    n_pairs, dim = C.c_int64(0), C.c_int32(0)
    check(lib().b2g_noise_pairs(C.byref(gemms.c), ket_size, ops_size, group_size, off.size, off.ctypes.data,
                                rows.ctypes.data, cols.ctypes.data, C.byref(pa), C.byref(n_pairs),
                                C.byref(dim)))
    return PairSeq({k: v[:n_pairs.value] for k, v in out.items()}), int(dim.value)


def with_identity(ops, id_dim: int) -> np.ndarray:
    """The operator blob followed by the row-major id_dim x id_dim identity."""
    ops = np.asarray(ops, dtype=np.float64)
    return np.concatenate([ops, np.eye(id_dim, dtype=np.float64).ravel()])


class PerturbativeNoise:
    """The perturbative-noise product of one converged ket on the device:
    ``noise(ket, group)`` adds it into ``group`` (device tensors or host
    arrays, as EffectiveHamiltonian.__call__ takes them)."""

    def __init__(self, ctx, gemms: GemmList, ops, ket_size: int, group_size: int, blk_off, blk_rows, blk_cols):
        from .heff import EffectiveHamiltonian
        ops = np.asarray(ops, dtype=np.float64)
        self.seq, self.id_dim = noise_pairs(gemms, ket_size, ops.size, group_size, blk_off, blk_rows, blk_cols)
        self.heff = EffectiveHamiltonian(ctx, self.seq, with_identity(ops, self.id_dim), ket_size, group_size)

    def __call__(self, ket, group, form: int = FP64):
        self.heff(ket, group, 1.0, form)

    def status(self):
        self.heff.status()

    def close(self):
        self.heff.close()
