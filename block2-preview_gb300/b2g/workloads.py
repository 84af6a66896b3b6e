"""Named H_eff workloads for benchmarking.

Each workload is one two-site effective Hamiltonian at the middle site of a
DMRG sweep, as recorded by the reference (its GEMM-pair sequence).  Small
ones carry the reference's own operator values (tests/golden); large ones
carry the reference's recorded structure only, with seeded synthetic operator
values of the same sizes (the throughput of H_eff*psi does not depend on the
values).
"""
from __future__ import annotations

import os

from .problem import HeffProblem, load_problem

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_ROOT = os.path.dirname(_PKG)
GOLDEN = os.path.join(_ROOT, "tests", "golden")

WORKLOADS = {
    "heff_hub16_su2_M250": os.path.join(GOLDEN, "hub16_su2_M250.npz"),
    "heff_syn8_su2_M60": os.path.join(GOLDEN, "syn8_su2.npz"),
    "heff_syn8_sz_M50": os.path.join(GOLDEN, "syn8_sz.npz"),
}
DEFAULT = "heff_hub16_su2_M250"


def get(name: str) -> HeffProblem:
    if name not in WORKLOADS:
        raise KeyError(f"unknown workload {name!r}; known: {sorted(WORKLOADS)}")
    p = load_problem(WORKLOADS[name])
    p.meta.setdefault("data", "reference operator values (golden fixture)")
    return p
