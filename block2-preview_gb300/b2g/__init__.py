"""GB300-native two-site DMRG hot path (block2's EffectiveHamiltonian H_eff*psi,
Davidson) behind the C ABI of include/b2g.h."""
from .capi import (B2GError, FP32, FP64, TF32X3, PairSeq, LIB_PATH, plan_stats, lib)  # noqa: F401
from .heff import Context, EffectiveHamiltonian  # noqa: F401
from .problem import HeffProblem, load_problem  # noqa: F401
