"""Container for one effective-Hamiltonian problem: the recorded pair
sequence, the operator blob, and (when known) psi / sigma / diag and the
converged Davidson results.  Stored as a compressed .npz."""
from __future__ import annotations

import json
from dataclasses import dataclass, field

import numpy as np

from .capi import PAIR_F64_FIELDS, PAIR_INT_FIELDS, PAIR_U64_FIELDS, PairSeq

PAIR_FIELDS = PAIR_INT_FIELDS + PAIR_F64_FIELDS + PAIR_U64_FIELDS


@dataclass
class HeffProblem:
    pairs: dict
    ops: np.ndarray
    psi_size: int
    sigma_size: int
    psi: np.ndarray | None = None
    sigma: np.ndarray | None = None
    diag: np.ndarray | None = None
    meta: dict = field(default_factory=dict)
    extra: dict = field(default_factory=dict)

    def seq(self) -> PairSeq:
        return PairSeq(self.pairs)

    @property
    def mnk(self) -> float:
        p = self.pairs
        return float(np.sum(p["m0"].astype(np.float64) * p["n0"] * p["k0"]
                            + p["m1"].astype(np.float64) * p["n1"] * p["k1"]))

    def save(self, path: str):
        d = {k: self.pairs[k] for k in PAIR_FIELDS}
        d["ops"] = self.ops
        for k in ("psi", "sigma", "diag"):
            v = getattr(self, k)
            if v is not None:
                d[k] = v
        for k, v in self.extra.items():
            d["x_" + k] = v
        meta = dict(self.meta, psi_size=self.psi_size, sigma_size=self.sigma_size)
        d["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(path, **d)


def load_problem(path: str) -> HeffProblem:
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    pairs = {k: z[k] for k in PAIR_FIELDS}
    get = lambda k: z[k] if k in z.files else None  # noqa: E731
    extra = {k[2:]: z[k] for k in z.files if k.startswith("x_")}
    return HeffProblem(pairs=pairs, ops=z["ops"], psi_size=int(meta["psi_size"]),
                       sigma_size=int(meta["sigma_size"]), psi=get("psi"), sigma=get("sigma"),
                       diag=get("diag"), meta=meta, extra=extra)
