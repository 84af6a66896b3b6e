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


_DUMP_DT = {"i4": np.int32, "u8": np.uint64, "f8": np.float64}


def load_dump(path: str) -> HeffProblem:
    """An H_eff written by the drop-in's dump (b2g_block2::HeffDump, raw
    arrays + manifest.txt): the translated pairs, the operator blob, the
    Davidson initial guess (psi), diag(H_eff) and the converged eigenvector."""
    import os

    arrays, scalars = {}, {}
    with open(os.path.join(path, "manifest.txt")) as f:
        for ln in f:
            t = ln.split()
            if not t:
                continue
            if t[0].startswith("#"):
                scalars[t[0][1:]] = float(t[1])
            else:
                arrays[t[0]] = np.fromfile(os.path.join(path, t[0] + ".bin"), dtype=_DUMP_DT[t[1]],
                                           count=int(t[2]))
    pairs = {k: arrays[k] for k in PAIR_FIELDS}
    extra = {}
    if "psi_converged" in arrays:
        extra["psi_converged"] = arrays["psi_converged"]
    return HeffProblem(pairs=pairs, ops=arrays["ops"], psi_size=int(scalars["psi_size"]),
                       sigma_size=int(scalars["sigma_size"]), psi=arrays.get("psi"),
                       diag=arrays.get("diag"), meta=dict(scalars), extra=extra)
