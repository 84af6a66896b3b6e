"""Generates tests/golden/*_cinfo.npz: the wavefunction connection infos of
one H_eff per case, with their inputs, written by the reference itself.

ConnectionInfo::initialize_wfn (src/core/sparse_matrix.hpp:163-292), called in
the EffectiveHamiltonian constructor (src/dmrg/effective_hamiltonian.hpp:
208-216), lists for every (conj type, operator sub-label) of H_eff and every
bra block the (left op block, right op block, ket block) triples that couple,
with their Clebsch-Gordan factor (a 9j symbol times transposition factors for
SU(2); 1 for SZ).  The harness (oracle/_ref/ref_harness) dumps the left/right
operator infos, the ket/bra block labels and the resulting connection infos
at the middle site of the named sweep.

Usage (needs the reference harness; not run on GPU machines):
    python tests/golden/make_cinfo_fixtures.py
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

from make_fixtures import CASES, HARNESS, RAW, fcidump_for, read_dump  # noqa: E402

KEYS = ("lop_dq", "lop_ferm", "lop_start", "lop_q", "rop_dq", "rop_ferm", "rop_start", "rop_q",
        "wfn_q", "bra_q", "cdq_vdq", "ci_opdq", "ci_n", "ci_q", "ci_qstart", "ci_idx", "ci_start",
        "ci_stride", "ci_factor", "ci_ia", "ci_ib", "ci_ic")


def main():
    for name in ("hub8_su2", "hub8_sz", "syn8_su2", "syn8_sz", "hub16_su2_M250"):
        args, desc = CASES[name]
        out = os.path.join(RAW, "cinfo", name)
        if os.path.exists(out):
            shutil.rmtree(out)
        os.makedirs(out)
        args = list(args)
        for i, a in enumerate(args):
            if a.startswith("@syn"):
                args[i] = fcidump_for(a[1:], out)
        cmd = [HARNESS, *args, "--seed", "1234", "--threads", "4", "--out", out]
        r = subprocess.run(cmd, capture_output=True, text=True,
                           env=dict(os.environ, OPENBLAS_NUM_THREADS="1"))
        if r.returncode != 0:
            raise RuntimeError(f"{name}: harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        (sd,) = [d for d in os.listdir(out) if d.startswith("sweep")]
        qa, qs = read_dump(os.path.join(out, sd, "qn"))
        path = os.path.join(HERE, name + "_cinfo.npz")
        np.savez_compressed(path, su2=np.int32(qs["su2"]), **{k: qa[k] for k in KEYS},
                            meta=np.array(json.dumps({"name": name + "_cinfo", "kind": "connection_info",
                                                      "description": "wavefunction connection infos of the "
                                                                     "H_eff at " + desc,
                                                      "harness_args": args + ["--seed", "1234"]})))
        print(f"{name}_cinfo: op infos {qa['lop_dq'].size}+{qa['rop_dq'].size}, "
              f"infos {qa['ci_opdq'].size}, entries {qa['ci_stride'].size} -> {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
