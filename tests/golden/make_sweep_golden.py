"""Records block2's own CPU sweep of the first benchmark configuration
(Hubbard L=16, t=1, U=4, half filling, S=0, SU(2), M=250; two warm-up sweeps
with noise 1e-6, 1e-7, then four sweeps at Davidson threshold 1e-10) as
tests/golden/sweep_hub16_su2_M250.json.  The run is oracle/_ref/dmrg_sweep_ref,
block2's DMRG::solve compiled from its sources by oracle/build_ref.sh.

    python tests/golden/make_sweep_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

from b2g.sweep import run_sweep  # noqa: E402
from test_sweep import HUB16  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "dmrg_sweep_ref")


def main():
    r = run_sweep(binary=REF_BIN, arms=("cpu",), threads=8, **HUB16)
    keep = {k: r[k] for k in ("n_sites", "threads", "seed", "const_e")}
    keep["config"] = {k: (list(v) if isinstance(v, tuple) else v) for k, v in HUB16.items()}
    for stage in ("warm",):
        keep[stage] = {k: v for k, v in r[stage].items() if k != "mps_blocks"}
    keep["arms"] = [r["arms"][0]]
    out = os.path.join(HERE, "sweep_hub16_su2_M250.json")
    with open(out, "w") as f:
        json.dump(keep, f, indent=1)
    print(out, r["arms"][0]["sweep_energies"])


if __name__ == "__main__":
    main()
