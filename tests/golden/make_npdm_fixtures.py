"""Generates tests/golden/*_npdm.npz: one site of the reference's PDM
expectation sweep (Expect with PDM1MPOQC / PDM2MPOQC on the final MPS of the
case, the fast algorithm TensorFunctions::tensor_product_expectation,
src/core/tensor_functions.hpp:1701-1877), recorded by the harness
(--pdm 1 --npdm-product C --npdm-order K) as

* GEMM pairs of the H_eff format (fields of b2g_pair_seq): "psi" holds the
  left operators, "ops" the ket (and the bra when it differs), and "sigma"
  the reference's partials <bra| a |ket> (block-transposed where p_trans);
* the partials' block layout (p_off, p_trans, p_nblk, b_off, b_rows, b_cols);
* the dot terms: expectation t_k gets t_f * dot(partial t_part, rmats[t_roff:
  t_roff + t_rsize]);
* the reference's expectation values of that site ("expect").

The harness runs with one thread, so the partials are recorded in one order.

Usage (needs the reference harness; not run on GPU machines):
    python tests/golden/make_npdm_fixtures.py [NAME]
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

# name -> (case whose final MPS is measured, PDM order, fast-expectation call recorded)
RUNS = {
    "hub8_su2_1pdm_npdm": ("hub8_su2", 1, 3),
    "hub8_sz_1pdm_npdm": ("hub8_sz", 1, 3),
    "syn8_su2_1pdm_npdm": ("syn8_su2", 1, 3),
    "hub8_su2_2pdm_npdm": ("hub8_su2", 2, 3),
    "syn8_sz_2pdm_npdm": ("syn8_sz", 2, 3),
}


def main():
    only = sys.argv[1] if len(sys.argv) > 1 else None
    for name, (case, order, call) in RUNS.items():
        if only and name != only:
            continue
        args, desc = CASES[case]
        out = os.path.join(RAW, "npdm", name)
        if os.path.exists(out):
            shutil.rmtree(out)
        os.makedirs(out)
        args = list(args)
        for i, a in enumerate(args):
            if a.startswith("@syn"):
                args[i] = fcidump_for(a[1:], out)
        extra = ["--seed", "1234", "--threads", "1", "--pdm", "1", "--npdm-product", str(call),
                 "--npdm-order", str(order)]
        r = subprocess.run([HARNESS, *args, *extra, "--out", out], capture_output=True, text=True,
                           env=dict(os.environ, OPENBLAS_NUM_THREADS="1"))
        if r.returncode != 0:
            raise RuntimeError(f"{name}: harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
        a, s = read_dump(os.path.join(out, "npdm_product"))
        meta = {"name": name, "kind": "pdm_fast_expectation",
                "description": "fast expectation %d of the %d-PDM sweep on the final MPS of %s" %
                               (call, order, desc),
                "harness_args": args + extra, "order": order,
                **{k: int(s[k]) for k in ("n_pairs", "n_partials", "n_expect", "n_terms", "psi_size",
                                          "ops_size", "sigma_size", "bra_is_ket")}}
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **a, meta=np.array(json.dumps(meta)))
        print(f"{name}: {meta['n_pairs']} pairs, {meta['n_partials']} partials "
              f"({int(np.sum(a['p_trans']))} transposed), {meta['n_expect']} expectations, "
              f"{meta['n_terms']} terms -> {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
