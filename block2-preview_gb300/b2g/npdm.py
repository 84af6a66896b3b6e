"""PDM expectations (block2's fast expectation algorithm) on the H_eff engine.

TensorFunctions::tensor_product_expectation (src/core/tensor_functions.hpp:1701-1877),
which Expect uses for the PDM MPOs, builds one partial <bra| a |ket> per unique
left operator a (OperatorFunctions::tensor_left_partial_expectation,
src/core/operator_functions.hpp:354-410), then takes every expectation as a sum
of factor * dot(partial, right operator).  Each partial block is one GEMM pair
of the H_eff format (work = a op2, partial (+)= op1^T work, with op1/op2 the
ket and bra blocks), so the partials of one site are one pair sequence: the
left operators play psi, the ket (and bra) blocks the operator blob, the
partials sigma.  A partial whose blocks come out transposed is stored
block-transposed; ``normal_layout`` undoes that before the dots.

``PdmSite`` runs the pairs on the device and takes the dots on the host.
"""
from __future__ import annotations

import numpy as np

from .capi import FP64, PairSeq


def normal_layout(partials, p_trans, p_nblk, b_off, b_rows, b_cols) -> np.ndarray:
    """The partials with every block of a transposed partial turned back to
    its row-major (rows x cols) layout."""
    out = np.array(partials, dtype=np.float64, copy=True)
    bi = 0
    for p in range(len(p_nblk)):
        for _ in range(int(p_nblk[p])):
            o, r, c = int(b_off[bi]), int(b_rows[bi]), int(b_cols[bi])
            bi += 1
            if p_trans[p]:
                out[o:o + r * c] = np.asarray(partials[o:o + r * c]).reshape(c, r).T.ravel()
    return out


def expectations(partials_normal, p_off, n_expect, t_k, t_part, t_roff, t_rsize, t_f, rmats) -> np.ndarray:
    """expect[k] = sum over the terms of k of factor * dot(partial, right
    operator), the last loops of tensor_product_expectation."""
    e = np.zeros(int(n_expect))
    for k, p, ro, rs, f in zip(t_k, t_part, t_roff, t_rsize, t_f):
        po, ro, rs = int(p_off[p]), int(ro), int(rs)
        e[int(k)] += f * float(partials_normal[po:po + rs] @ rmats[ro:ro + rs])
    return e


class PdmSite:
    """The fast expectation of one site: ``values(form)`` runs the partials'
    pairs on the device and returns the expectation values."""

    def __init__(self, ctx, seq: PairSeq, left_ops, wfn, sigma_size: int, layout: dict, terms: dict,
                 rmats, n_expect: int):
        from .heff import EffectiveHamiltonian
        self.left_ops = np.ascontiguousarray(left_ops, dtype=np.float64)
        self.sigma_size = int(sigma_size)
        self.layout, self.terms = layout, terms
        self.rmats = np.ascontiguousarray(rmats, dtype=np.float64)
        self.n_expect = int(n_expect)
        self.heff = EffectiveHamiltonian(ctx, seq, wfn, self.left_ops.size, self.sigma_size)

    def partials(self, form: int = FP64) -> np.ndarray:
        """The partials in their storage layout (host copy)."""
        out = np.zeros(self.sigma_size)
        self.heff(self.left_ops, out, 1.0, form)
        self.heff.status()
        return out

    def values(self, form: int = FP64) -> np.ndarray:
        L, T = self.layout, self.terms
        normal = normal_layout(self.partials(form), L["p_trans"], L["p_nblk"], L["b_off"], L["b_rows"],
                               L["b_cols"])
        return expectations(normal, L["p_off"], self.n_expect, T["t_k"], T["t_part"], T["t_roff"],
                            T["t_rsize"], T["t_f"], self.rmats)

    def close(self):
        self.heff.close()
