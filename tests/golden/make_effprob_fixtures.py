"""Generates tests/golden/*_effprob.npz: the reference's own EffectiveProblem
export (EFFPROB1 file, EffectiveHamiltonian::save_eff_problem,
src/dmrg/effective_hamiltonian.hpp:254-261) of one H_eff per case, with the
wavefunction connection infos and block lists the harness dumps from the same
H_eff object in the same run (the fields b2g.effprob must decode to).

Usage (needs the reference harness; not run on GPU machines):
    python tests/golden/make_effprob_fixtures.py
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_cinfo_fixtures import KEYS  # noqa: E402
from make_fixtures import CASES, HARNESS, RAW, fcidump_for, read_dump  # noqa: E402

QN_KEYS = ("wfn_q", "wfn_rows", "wfn_cols", "wfn_shift", "dq_target")


def main():
    for name in ("hub8_su2", "hub8_sz", "syn8_su2", "syn8_sz"):
        args, desc = CASES[name]
        out = os.path.join(RAW, "effprob", name)
        if os.path.exists(out):
            shutil.rmtree(out)
        os.makedirs(out)
        args = list(args)
        for i, a in enumerate(args):
            if a.startswith("@syn"):
                args[i] = fcidump_for(a[1:], out)
        cmd = [HARNESS, *args, "--seed", "1234", "--threads", "4", "--effprob", "1", "--out", out]
        r = subprocess.run(cmd, capture_output=True, text=True,
                           env=dict(os.environ, OPENBLAS_NUM_THREADS="1"))
        if r.returncode != 0:
            raise RuntimeError(f"{name}: harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        (sd,) = [d for d in os.listdir(out) if d.startswith("sweep")]
        qn = os.path.join(out, sd, "qn")
        qa, qs = read_dump(qn)
        with open(os.path.join(qn, "effprob.bin"), "rb") as f:
            raw = np.frombuffer(f.read(), dtype=np.uint8)
        path = os.path.join(HERE, name + "_effprob.npz")
        np.savez_compressed(
            path, effprob=raw, su2=np.int32(qs["su2"]), isite=np.int32(qs["effprob_isite"]),
            forward=np.int32(qs["effprob_forward"]), **{k: qa[k] for k in KEYS + QN_KEYS},
            meta=np.array(json.dumps({"name": name + "_effprob", "kind": "effective_problem_export",
                                      "description": "the reference's EFFPROB1 export of the H_eff at " + desc,
                                      "harness_args": args + ["--seed", "1234", "--effprob", "1"]})))
        print(f"{name}_effprob: {raw.size} bytes of EFFPROB1, {qa['ci_opdq'].size} connection infos "
              f"-> {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
