"""Host-side mirror of block2's environment blocking for the GB300 path.

TensorFunctions::left_contract / right_contract (src/core/tensor_functions.hpp:
2842-2986) build the enlarged block's operators; at block level that is a list
of iadd records (sums of operators, OperatorFunctions::iadd,
src/core/operator_functions.hpp:135-170) and Kronecker records
(OperatorFunctions::tensor_product, operator_functions.hpp:672-710).
``contract`` replays such a record list on the GPU (b2g_block_contract).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .capi import BlockSeqC, check, lib

IADD_FIELDS = {"ia_m": np.int32, "ia_n": np.int32, "ia_conj": np.int32, "ia_src_blob": np.int32,
               "ia_dst": np.uint64, "ia_src": np.uint64, "ia_f": np.float64}
KRON_FIELDS = {"kr_am": np.int32, "kr_an": np.int32, "kr_ca": np.int32, "kr_bm": np.int32,
               "kr_bn": np.int32, "kr_cb": np.int32, "kr_cn": np.int32, "kr_ablob": np.int32,
               "kr_bblob": np.int32, "kr_a": np.uint64, "kr_b": np.uint64, "kr_c": np.uint64,
               "kr_f": np.float64}


class BlockSeq:
    """The record arrays (dict-like input with the IADD_FIELDS and KRON_FIELDS keys)."""

    def __init__(self, arrays):
        self.arrays = {}
        for k, dt in {**IADD_FIELDS, **KRON_FIELDS}.items():
            self.arrays[k] = np.ascontiguousarray(arrays[k], dtype=dt)
        self.n_iadd = self.arrays["ia_m"].size
        self.n_kron = self.arrays["kr_am"].size
        a = self.arrays
        self.c = BlockSeqC(self.n_iadd, *[a[k].ctypes.data for k in ("ia_m", "ia_n", "ia_conj", "ia_src_blob",
                                                                     "ia_dst", "ia_src", "ia_f")],
                           self.n_kron, *[a[k].ctypes.data for k in KRON_FIELDS])


def contract(ctx, seq, env, site, tmp_size: int, out_size: int) -> np.ndarray:
    """The enlarged block's operator data (out_size doubles) from env and site."""
    if not isinstance(seq, BlockSeq):
        seq = BlockSeq(seq)
    env = np.ascontiguousarray(env, dtype=np.float64)
    site = np.ascontiguousarray(site, dtype=np.float64)
    out = np.zeros(max(int(out_size), 1))
    check(lib().b2g_block_contract(ctx.handle, C.byref(seq.c), env.ctypes.data, env.size, site.ctypes.data,
                                   site.size, int(tmp_size), out.ctypes.data, int(out_size)))
    return out[:int(out_size)]


def contract_device(ctx, seq, env, site, tmp_size: int, out):
    """Device-resident blocking: env, site and out are contiguous float64 CUDA
    tensors (out holds out.numel() doubles and is overwritten)."""
    if not isinstance(seq, BlockSeq):
        seq = BlockSeq(seq)
    for t in (env, site, out):
        if not (t.is_cuda and t.is_contiguous()):
            raise TypeError("env, site and out must be contiguous CUDA tensors")
    check(lib().b2g_block_contract_device(ctx.handle, C.byref(seq.c), env.data_ptr(), env.numel(),
                                          site.data_ptr(), site.numel(), int(tmp_size), out.data_ptr(),
                                          out.numel()))
    return out
