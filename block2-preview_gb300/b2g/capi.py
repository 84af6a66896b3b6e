"""ctypes binding of the C ABI in include/b2g.h (libb2g.so).

The library is the only compute path: importing this module on a machine
where lib/libb2g.so has not been built raises, it never falls back to a CPU
implementation.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libb2g.so")

B2G_OK = 0
B2G_ERR_ARG = 1
B2G_ERR_CUDA = 2
B2G_ERR_NOMEM = 3
B2G_ERR_UNSUPPORTED = 4
B2G_ERR_NOT_CONVERGED = 5
B2G_ERR_STATE = 6

FP64 = 0
TF32X3 = 1
FP32 = 2
PROBE_FP64_MMA = 16  # b2g_probe_peak only: the FP64 tensor-core instruction (DMMA)

_i32p = C.POINTER(C.c_int32)
_u64p = C.POINTER(C.c_uint64)
_f64p = C.POINTER(C.c_double)


class PairSeqC(C.Structure):
    """b2g_pair_seq: the recorded GEMM-pair sequence (struct of arrays)."""

    _fields_ = [
        ("n_pairs", C.c_int64),
        ("tb0", _i32p), ("m0", _i32p), ("n0", _i32p), ("k0", _i32p), ("lda0", _i32p), ("ldb0", _i32p),
        ("ta1", _i32p), ("m1", _i32p), ("n1", _i32p), ("k1", _i32p), ("lda1", _i32p), ("ldc1", _i32p),
        ("alpha0", _f64p), ("alpha1", _f64p),
        ("a0", _u64p), ("b0", _u64p), ("a1", _u64p), ("c1", _u64p),
    ]


class HeffStatsC(C.Structure):
    _fields_ = [
        ("n_pairs", C.c_int64), ("n_work", C.c_int64), ("n_regions", C.c_int64), ("n_tiles", C.c_int64),
        ("mnk", C.c_double), ("mnk_executed", C.c_double),
        ("ops_bytes", C.c_uint64), ("work_bytes", C.c_uint64), ("plan_bytes", C.c_uint64),
        ("psi_size", C.c_uint64), ("sigma_size", C.c_uint64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class DavidsonResultC(C.Structure):
    _fields_ = [
        ("energy", C.c_double), ("n_iter", C.c_int32), ("n_apply_fp64", C.c_int32),
        ("n_apply_mixed", C.c_int32), ("residual_norm2", C.c_double),
    ]


class TuneResultC(C.Structure):
    _fields_ = [
        ("n_candidates", C.c_int32), ("best", C.c_int32), ("ms", C.c_float * 12),
        ("g0_tile_cols", C.c_int32 * 12), ("g1_tile_cols", C.c_int32 * 12), ("g1_chunk", C.c_int32 * 12),
        ("g1_wide_frac", C.c_double), ("g0_wide_frac", C.c_double),
    ]

    def as_dict(self):
        n = self.n_candidates
        return {"best": self.best,
                "candidates": [{"g0_tile_cols": self.g0_tile_cols[i], "g1_tile_cols": self.g1_tile_cols[i],
                                "g1_chunk": self.g1_chunk[i], "ms": float(self.ms[i])} for i in range(n)],
                "g1_wide_frac": self.g1_wide_frac, "g0_wide_frac": self.g0_wide_frac}


class GemmListC(C.Structure):
    """b2g_gemm_list: the single GEMMs of a perturbative-noise product."""

    _fields_ = [("n_gemms", C.c_int64)] + [(k, _i32p) for k in ("ta", "tb", "m", "n", "k", "lda", "ldb", "ldc",
                                                               "a_kind", "b_kind")] + \
               [("alpha", _f64p), ("beta", _f64p), ("a", _u64p), ("b", _u64p), ("c", _u64p)]


class PairArraysC(C.Structure):
    """b2g_pair_arrays: writable pair arrays (the fields of b2g_pair_seq)."""

    _fields_ = [(k, _i32p) for k in ("tb0", "m0", "n0", "k0", "lda0", "ldb0", "ta1", "m1", "n1", "k1",
                                     "lda1", "ldc1")] + \
               [("alpha0", _f64p), ("alpha1", _f64p), ("a0", _u64p), ("b0", _u64p), ("a1", _u64p), ("c1", _u64p)]


class DmLayoutC(C.Structure):
    _fields_ = [
        ("trace_right", C.c_int32), ("n_psi_blocks", C.c_int32), ("psi_dm", C.c_void_p),
        ("psi_rows", C.c_void_p), ("psi_cols", C.c_void_p), ("psi_off", C.c_void_p),
        ("n_dm_blocks", C.c_int32), ("dm_dim", C.c_void_p),
    ]


class DmResultC(C.Structure):
    _fields_ = [("error", C.c_double), ("n_kept", C.c_int32)]


class BlockSeqC(C.Structure):
    _fields_ = [
        ("n_iadd", C.c_int64), ("ia_m", C.c_void_p), ("ia_n", C.c_void_p), ("ia_conj", C.c_void_p),
        ("ia_src_blob", C.c_void_p), ("ia_dst", C.c_void_p), ("ia_src", C.c_void_p), ("ia_f", C.c_void_p),
        ("n_kron", C.c_int64), ("kr_am", C.c_void_p), ("kr_an", C.c_void_p), ("kr_ca", C.c_void_p),
        ("kr_bm", C.c_void_p), ("kr_bn", C.c_void_p), ("kr_cb", C.c_void_p), ("kr_cn", C.c_void_p),
        ("kr_ablob", C.c_void_p), ("kr_bblob", C.c_void_p), ("kr_a", C.c_void_p), ("kr_b", C.c_void_p),
        ("kr_c", C.c_void_p), ("kr_f", C.c_void_p),
    ]


# every symbol declared in include/b2g.h, with its ctypes signature
SIGNATURES = {
    "b2g_version": (C.c_int, []),
    "b2g_last_error": (C.c_char_p, []),
    "b2g_context_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "b2g_context_destroy": (C.c_int, [C.c_void_p]),
    "b2g_context_stream": (C.c_void_p, [C.c_void_p]),
    "b2g_context_synchronize": (C.c_int, [C.c_void_p]),
    "b2g_heff_create": (C.c_int, [C.c_void_p, C.POINTER(PairSeqC), C.c_void_p, C.c_uint64, C.c_int,
                                  C.c_uint64, C.c_uint64, C.POINTER(C.c_void_p)]),
    "b2g_heff_destroy": (C.c_int, [C.c_void_p]),
    "b2g_heff_status": (C.c_int, [C.c_void_p]),
    "b2g_heff_stats_get": (C.c_int, [C.c_void_p, C.POINTER(HeffStatsC)]),
    "b2g_plan_stats": (C.c_int, [C.POINTER(PairSeqC), C.c_uint64, C.c_uint64, C.c_uint64,
                                 C.POINTER(HeffStatsC)]),
    "b2g_partition_pairs": (C.c_int, [C.POINTER(PairSeqC), C.c_int, C.c_void_p, C.c_void_p]),
    "b2g_heff_apply": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int]),
    "b2g_heff_apply_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int]),
    "b2g_heff_apply_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                       C.c_int]),
    "b2g_heff_diag": (C.c_int, [C.c_void_p, C.c_void_p]),
    "b2g_block_contract": (C.c_int, [C.c_void_p, C.POINTER(BlockSeqC), C.c_void_p, C.c_uint64, C.c_void_p,
                                     C.c_uint64, C.c_uint64, C.c_void_p, C.c_uint64]),
    "b2g_block_contract_device": (C.c_int, [C.c_void_p, C.POINTER(BlockSeqC), C.c_void_p, C.c_uint64, C.c_void_p,
                                     C.c_uint64, C.c_uint64, C.c_void_p, C.c_uint64]),
    "b2g_heff_diag_host": (C.c_int, [C.c_void_p, C.c_void_p]),
    "b2g_heff_apply_noalloc": (C.c_int, [C.POINTER(PairSeqC), C.c_void_p, C.c_uint64, C.c_void_p,
                                         C.c_uint64, C.c_void_p, C.c_uint64, C.c_double, C.c_void_p]),
    "b2g_heff_set_ops": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "b2g_heff_adjoint_prepare": (C.c_int, [C.c_void_p, C.POINTER(PairSeqC)]),
    "b2g_heff_adjoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                                   C.c_void_p]),
    "b2g_heff_adjoint_mnk": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "b2g_heff_set_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "b2g_heff_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "b2g_heff_graph_count": (C.c_int, [C.c_void_p]),
    "b2g_heff_autotune": (C.c_int, [C.c_void_p, C.POINTER(PairSeqC), C.c_int, C.POINTER(TuneResultC)]),
    "b2g_heff_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "b2g_heff_set_params": (C.c_int, [C.c_void_p, C.POINTER(PairSeqC), C.c_void_p]),
    "b2g_heff_last_timing": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "b2g_probe_peak": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "b2g_launch_count": (C.c_int, [C.POINTER(C.c_uint64)]),
    "b2g_host_buffer": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "b2g_davidson": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int,
                               C.c_int, C.c_int, C.POINTER(DavidsonResultC)]),
    "b2g_davidson_multi": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                                     C.c_int, C.c_int, C.c_int, C.c_void_p, C.POINTER(DavidsonResultC)]),
    "b2g_quanta_op": (C.c_int, [C.c_int, C.c_int, C.c_uint64, C.c_uint64, C.c_uint64,
                                C.POINTER(C.c_uint64)]),
    "b2g_state_tensor_product": (C.c_int, [C.c_int, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_uint64, C.c_void_p]),
    "b2g_state_connection": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "b2g_wfn_blocks": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_uint64, C.c_int, C.c_uint32,
                                 C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                 C.POINTER(C.c_int), C.POINTER(C.c_uint32)]),
    "b2g_wfn_connection": (C.c_int, [C.c_int, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int32, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "b2g_noise_pairs": (C.c_int, [C.POINTER(GemmListC), C.c_uint64, C.c_uint64, C.c_uint64, C.c_int64,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(PairArraysC),
                                  C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "b2g_dm_truncate": (C.c_int, [C.c_void_p, C.POINTER(DmLayoutC), C.c_void_p, C.c_int, C.c_double,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.POINTER(DmResultC)]),
}

_lib = None


class B2GError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"b2g error {code}: {msg}")
        self.code = code


def lib():
    """Load libb2g.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with build.build() "
                              "(nvcc, sm_103a); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != B2G_OK:
        msg = lib().b2g_last_error()
        raise B2GError(rc, msg.decode() if msg else "")
    return rc


PAIR_INT_FIELDS = ("tb0", "m0", "n0", "k0", "lda0", "ldb0", "ta1", "m1", "n1", "k1", "lda1", "ldc1")
PAIR_F64_FIELDS = ("alpha0", "alpha1")
PAIR_U64_FIELDS = ("a0", "b0", "a1", "c1")


class PairSeq:
    """Owns numpy arrays of a recorded pair sequence and exposes the C struct.

    ``arrays`` maps the field names of b2g_pair_seq to 1-D arrays of equal
    length (converted to int32 / float64 / uint64 contiguous copies).
    """

    def __init__(self, arrays):
        n = len(arrays["m0"])
        self.arrays = {}
        for k in PAIR_INT_FIELDS:
            self.arrays[k] = np.ascontiguousarray(arrays[k], dtype=np.int32)
        for k in PAIR_F64_FIELDS:
            self.arrays[k] = np.ascontiguousarray(arrays[k], dtype=np.float64)
        for k in PAIR_U64_FIELDS:
            self.arrays[k] = np.ascontiguousarray(arrays[k], dtype=np.uint64)
        for k, v in self.arrays.items():
            if v.shape != (n,):
                raise ValueError(f"pair field {k} has shape {v.shape}, expected ({n},)")
        self.n = n
        s = PairSeqC()
        s.n_pairs = n
        for k in PAIR_INT_FIELDS:
            setattr(s, k, self.arrays[k].ctypes.data_as(_i32p))
        for k in PAIR_F64_FIELDS:
            setattr(s, k, self.arrays[k].ctypes.data_as(_f64p))
        for k in PAIR_U64_FIELDS:
            setattr(s, k, self.arrays[k].ctypes.data_as(_u64p))
        self.c = s

    def subset(self, idx) -> "PairSeq":
        """The pairs at positions idx (in that order) as a new sequence."""
        idx = np.asarray(idx, dtype=np.int64)
        return PairSeq({k: v[idx] for k, v in self.arrays.items()})

    def transposed(self) -> "PairSeq":
        """The pairs of H_eff^T: pair i becomes W = x[c1:] op_b0(ops[b0:])^T,
        out[a0:] += alpha op_a1(ops[a1:])^T W (both operator flags flipped, the
        psi and sigma roles swapped), so applying it to x gives H_eff^T x."""
        a = self.arrays
        return PairSeq({"tb0": 1 - a["tb0"], "m0": a["m1"], "k0": a["n1"], "n0": a["k0"],
                        "lda0": a["ldc1"], "ldb0": a["ldb0"], "a0": a["c1"], "b0": a["b0"],
                        "ta1": 1 - a["ta1"], "m1": a["m0"], "k1": a["m1"], "n1": a["k0"],
                        "lda1": a["lda1"], "ldc1": a["lda0"], "a1": a["a1"], "c1": a["a0"],
                        "alpha0": a["alpha0"], "alpha1": a["alpha1"]})

    def symmetrized(self) -> "PairSeq":
        """The pairs of (H_eff + H_eff^T) / 2 (square H_eff only)."""
        t = self.transposed()
        both = {k: np.concatenate([self.arrays[k], t.arrays[k]]) for k in self.arrays}
        both["alpha1"] = both["alpha1"] * 0.5
        return PairSeq(both)

    def mnk(self) -> float:
        a = self.arrays
        return float(np.sum(a["m0"].astype(np.float64) * a["n0"] * a["k0"]
                            + a["m1"].astype(np.float64) * a["n1"] * a["k1"]))


def plan_stats(seq: PairSeq, ops_size: int, psi_size: int, sigma_size: int) -> dict:
    st = HeffStatsC()
    check(lib().b2g_plan_stats(C.byref(seq.c), ops_size, psi_size, sigma_size, C.byref(st)))
    return st.as_dict()
