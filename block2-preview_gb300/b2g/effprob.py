"""Reader of the reference's EffectiveProblem export (EFFPROB1 files).

block2 can export one effective Hamiltonian as a file
(EffectiveHamiltonian::save_eff_problem, src/dmrg/effective_hamiltonian.hpp:
254-261, format src/core/effective_problem.hpp:72-247, version 2): a header,
the symbolic operator tensor of H_eff (the left/right operator tensors with
their symbolic matrices, operator expressions and operator matrix infos, and
for a delayed tensor its delayed expressions and the expressions' slots),
the metadata of the bra/ket wavefunctions, the operator delta quantum, and
per operator quantum the wavefunction connection info with its CG factors.
Operator matrices of the normal type carry only their size (the values live
in block2's operator files); delayed ones carry their operator expression.

``read_effective_problem(path)`` returns nested dicts of plain Python values
and numpy arrays; expressions are dicts with a ``type`` key ("elem", "prod",
"sum", "sumprod", "elemref", "exprref", "zero").  The layouts are those of
the reference's default build (8-byte quantum labels, 16-bit ubond_t, FP64,
real); other builds are rejected.  The connection infos are the objects this
library restates in b2g_wfn_connection; the reader checks them against the
reference's dumps (tests/test_effprob.py).
"""
from __future__ import annotations

import struct

import numpy as np

from .mps_io import FormatError

MAGIC = b"EFFPROB1"
SYMMETRIES = {1: "SU2", 2: "SZ", 3: "SU2K", 4: "SZK", 5: "SGF", 6: "SGB", 7: "SAny"}
OP_TYPES = {0: "zero", 1: "elem", 2: "prod", 3: "sum", 4: "elemref", 5: "sumprod", 6: "exprref"}
SYM_TYPES = {0: "rvec", 1: "cvec", 2: "mat"}
MATRIX_TYPES = {0: "normal", 1: "csr", 2: "archived", 3: "delayed"}


class _Stream:
    def __init__(self, buf: bytes):
        self.buf, self.pos = buf, 0

    def take(self, n: int) -> bytes:
        if n < 0 or self.pos + n > len(self.buf):
            raise FormatError(f"truncated EFFPROB file at byte {self.pos} (wanted {n})")
        b = self.buf[self.pos:self.pos + n]
        self.pos += n
        return b

    def unpack(self, fmt: str):
        return struct.unpack("<" + fmt, self.take(struct.calcsize("<" + fmt)))

    def one(self, fmt: str):
        return self.unpack(fmt)[0]

    def array(self, dtype: str, n: int) -> np.ndarray:
        dt = np.dtype(dtype)
        return np.frombuffer(self.take(dt.itemsize * n), dt).copy()


def _expr(s: _Stream) -> dict:
    tp = s.one("B")
    kind = OP_TYPES.get(tp)
    if kind is None:
        raise FormatError(f"unknown operator expression type {tp}")
    if kind == "zero":
        return {"type": "zero"}
    if kind == "elem":
        name, site, factor, q = s.unpack("BQdQ")
        return {"type": "elem", "name": name, "site_index": site, "factor": factor, "q_label": q}
    if kind == "elemref":
        factor, trans = s.unpack("bb")
        return {"type": "elemref", "factor": factor, "trans": trans, "op": _expr(s)}
    if kind == "prod":
        factor, conj, has = s.unpack("dBB")
        return {"type": "prod", "factor": factor, "conj": conj,
                "a": _expr(s) if has & 1 else None, "b": _expr(s) if has & 2 else None}
    if kind == "sum":
        n = s.one("i")
        return {"type": "sum", "strings": [_expr(s) for _ in range(n)]}
    if kind == "sumprod":
        factor, conj, has = s.unpack("dBB")
        a = _expr(s) if has & 1 else None
        b = _expr(s) if has & 2 else None
        c = _expr(s) if has & 4 else None
        n = s.one("i")
        ops = [_expr(s) for _ in range(n)]
        conjs = [bool(x) for x in s.array("u1", n)]
        return {"type": "sumprod", "factor": factor, "conj": conj, "a": a, "b": b, "c": c, "ops": ops,
                "conjs": conjs}
    # exprref
    is_local = bool(s.one("B"))
    op = _expr(s)
    has_orig = s.one("B")
    return {"type": "exprref", "is_local": is_local, "op": op, "orig": _expr(s) if has_orig & 1 else None}


def _symbolic(s: _Stream) -> dict:
    tp, m, n, sz = s.unpack("Biii")
    kind = SYM_TYPES.get(tp)
    if kind is None:
        raise FormatError(f"unknown symbolic tensor type {tp}")
    data = [_expr(s) for _ in range(sz)]
    out = {"type": kind, "m": m, "n": n, "data": data}
    if kind == "mat":
        out["indices"] = s.array("<i4", 2 * sz).reshape(sz, 2)
    return out


def _matrix_info(s: _Stream) -> dict:
    dq, n = s.unpack("Qi")
    if n < 0:
        raise FormatError("negative block count in a SparseMatrixInfo")
    info = {"delta_quantum": dq, "quanta": s.array("<u8", n), "n_states_bra": s.array("<u2", n),
            "n_states_ket": s.array("<u2", n), "block_shifts": s.array("<u4", n)}
    info["is_fermion"], info["flags"] = s.unpack("BB")
    return info


def _connection_info(s: _Stream) -> dict:
    n = s.array("<i4", 5)
    nc = s.one("i")
    ci = {"n": n, "nc": nc}
    ci["quanta"] = s.array("<u8", int(n[4]))
    ci["idx"] = s.array("<u4", int(n[4]))
    ci["stride"] = s.array("<u8", nc)
    ci["factor"] = s.array("<f8", nc)
    ci["ia"], ci["ib"], ci["ic"] = s.array("<u4", nc), s.array("<u4", nc), s.array("<u4", nc)
    return ci


def _operator_matrix(s: _Stream) -> dict:
    tp = s.one("B")
    kind = MATRIX_TYPES.get(tp)
    if kind is None:
        raise FormatError(f"unknown operator matrix type {tp}")
    m = {"type": kind, "info": _matrix_info(s)}
    m["cinfo"] = _connection_info(s) if s.one("B") else None
    if kind == "normal":
        m["total_memory"] = s.one("Q")
    elif kind == "delayed":
        # a delayed site operator: its site count and operator expression
        m["m"] = s.one("H")
        m["op"] = _expr(s)
    else:
        raise FormatError(f"{kind} operator matrices are not supported by this reader")
    return m


def _operator_tensor(s: _Stream):
    if not s.one("B"):
        return None
    tag = s.one("B")
    if tag not in (0, 1):
        raise FormatError(f"unknown operator tensor tag {tag}")
    lr = s.one("B")
    t = {"delayed": tag == 1, "lr": lr, "lmat": None, "rmat": None}
    if lr in (1, 2):
        t["lmat"] = _symbolic(s)
        if lr == 1:
            t["rmat"] = t["lmat"]          # one symbolic matrix for both sides
    elif lr == 3:
        t["rmat"] = _symbolic(s)
    elif lr == 0:
        t["lmat"], t["rmat"] = _symbolic(s), _symbolic(s)
    elif lr != 4:
        raise FormatError(f"unknown symbolic-matrix layout {lr}")
    t["ops"] = [(_expr(s), _operator_matrix(s)) for _ in range(s.one("i"))]
    if t["delayed"]:
        t["dops"] = [_expr(s) for _ in range(s.one("i"))]
        t["mat"] = _symbolic(s) if s.one("B") else None
        t["stacked_mat"] = _symbolic(s) if s.one("B") else None
        t["lopt"] = _operator_tensor(s)
        t["ropt"] = _operator_tensor(s)
        t["exprs"] = []
        for _ in range(s.one("i")):
            e = _expr(s)
            slot, value = s.unpack("Qd")
            t["exprs"].append((e, slot, value))
    return t


def _matrix_metadata(s: _Stream):
    if not s.one("B"):
        return None
    tp = s.one("B")
    info = _matrix_info(s)
    factor, total = s.unpack("dQ")
    return {"type": MATRIX_TYPES.get(tp, tp), "info": info, "factor": factor, "total_memory": total}


def read_effective_problem(path: str) -> dict:
    """Parses one EFFPROB1 file written by the reference."""
    with open(path, "rb") as f:
        s = _Stream(f.read())
    if s.take(8) != MAGIC:
        raise FormatError("not an EFFPROB1 file")
    version, symm = s.unpack("IB")
    if version != 2:
        raise FormatError(f"EFFPROB version {version} (this reader knows version 2)")
    q_size, fl_size, fp_size, cpx, ubond, align = s.unpack("BBBBBB")
    if (q_size, fl_size, fp_size, cpx, ubond) != (8, 8, 8, 1, 2):
        raise FormatError("only the reference's default build is read (8-byte labels, real FP64, "
                          "16-bit ubond_t)")
    isite, forward = s.unpack("iB")
    out = {"version": version, "symmetry": SYMMETRIES.get(symm, symm), "align_type": align, "isite": isite,
           "forward": bool(forward)}
    out["op"] = _operator_tensor(s)
    out["cmat"] = _matrix_metadata(s)
    out["vmat"] = _matrix_metadata(s)
    out["opdq"] = s.one("Q")
    terms = []
    for _ in range(s.one("i")):
        q = s.one("Q")
        terms.append({"operator_quantum": q, "cinfo": _connection_info(s) if s.one("B") else None})
    out["terms"] = terms
    if s.pos != len(s.buf):
        raise FormatError(f"{len(s.buf) - s.pos} trailing bytes after the connection infos")
    return out
