"""Generates tests/golden/*_noise.npz: the reference's perturbative-noise
product of one converged two-site wavefunction per case
(EffectiveHamiltonian::perturbative_noise with NoiseTypes::ReducedPerturbative,
Perturbative or ReducedPerturbativeLowMem,
src/dmrg/effective_hamiltonian.hpp:262-433, requested the way
DMRG::two_dot_eigs_and_perturb does, src/dmrg/sweep_algorithm.hpp:1257-1260),
recorded by the harness (--noise-product 1): the single GEMMs block2 records
in Tasked mode (g_* arrays, the fields of b2g_gemm_list), the operator blob
they read, the converged ket ("psi"), the reference's perturbed wavefunction
group ("sigma") and the group's block layout (blk_rows/blk_cols/blk_off/blk_vec,
vec_q).

The harness runs with one thread: the recorder reads the GEMMs from the one
sequence they are recorded into.

Usage (needs the reference harness; not run on GPU machines):
    python tests/golden/make_noise_fixtures.py [NAME]
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

LAYOUT = ("vec_q", "blk_rows", "blk_cols", "blk_off", "blk_vec")
# name -> (case the run follows, sweep whose middle site is dumped, NoiseTypes value);
# an even sweep runs forward (op(L) psi), an odd one backward (psi op(R));
# 12 = ReducedPerturbative, 4 = Perturbative (one vector per perturbation),
# 76 = ReducedPerturbativeLowMem
RUNS = {
    "hub8_su2_noise": ("hub8_su2", 0, 12),
    "hub8_su2_bw_noise": ("hub8_su2", 1, 12),
    "hub8_sz_noise": ("hub8_sz", 0, 12),
    "syn8_su2_noise": ("syn8_su2", 1, 12),
    "syn8_sz_fw_noise": ("syn8_sz", 0, 12),
    "syn8_sz_noise": ("syn8_sz", 1, 12),
    "hub8_su2_full_noise": ("hub8_su2", 0, 4),
    "syn8_su2_full_noise": ("syn8_su2", 1, 4),
    "syn8_sz_lowmem_noise": ("syn8_sz", 1, 76),
}


def main():
    only = sys.argv[1] if len(sys.argv) > 1 else None
    for name, (case, sweep, noise) in RUNS.items():
        if only and name != only:
            continue
        args, desc = CASES[case]
        out = os.path.join(RAW, "noise", name)
        if os.path.exists(out):
            shutil.rmtree(out)
        os.makedirs(out)
        args = list(args)
        for i, a in enumerate(args):
            if a.startswith("@syn"):
                args[i] = fcidump_for(a[1:], out)
        args[args.index("--dump-sweep") + 1] = str(sweep)
        cmd = [HARNESS, *args, "--seed", "1234", "--threads", "1", "--noise-product", str(noise), "--out", out]
        r = subprocess.run(cmd, capture_output=True, text=True, env=dict(os.environ, OPENBLAS_NUM_THREADS="1"))
        if r.returncode != 0:
            raise RuntimeError(f"{name}: harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        (sd,) = [d for d in os.listdir(out) if d.startswith("sweep")]
        a, s = read_dump(os.path.join(out, sd, "noise"))
        n_left = int(np.sum(a["g_akind"] == 0))
        meta = {"name": name, "kind": "perturbative_noise",
                "description": "perturbative-noise product (NoiseTypes %d) of the converged "
                               "ket at the middle site of sweep %d (%s) of %s" %
                               (noise, sweep, "forward" if int(s["forward"]) else "backward", desc),
                "harness_args": args + ["--seed", "1234", "--threads", "1", "--noise-product", str(noise)],
                "noise_type": int(s["noise_type"]),
                "n_gemms": int(s["n_gemms"]), "n_ket_left": n_left, "n_ket_right": int(s["n_gemms"]) - n_left,
                "n_held": int(s["n_held"]), "forward": int(s["forward"]), "n_vectors": int(s["n_vectors"]),
                "psi_size": int(s["psi_size"]), "sigma_size": int(s["sigma_size"])}
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **a, meta=np.array(json.dumps(meta)))
        print(f"{name}: {meta['n_gemms']} GEMMs (ket left {n_left}, right {meta['n_ket_right']}, "
              f"held {meta['n_held']}), {meta['n_vectors']} vectors, ops {a['ops'].size} "
              f"-> {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
