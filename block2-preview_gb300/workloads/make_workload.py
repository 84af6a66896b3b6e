"""Packs one recorded H_eff structure (a site directory dumped by
oracle/ref_harness with --with-data 0) into a workload file for bench.py.

Usage: python make_workload.py DUMP_SITE_DIR OUT.npz "description"

The structure files committed beside this script were made from these
reference runs (synthetic integrals of b2g.integrals, seed 0):
  heff_syn24_su2_M1000_sweep0.npz: n=24 N=24 SU(2) M=1000, sweep 0 middle site
      ref_harness --ham syn_n24.FCIDUMP --M 1000 --sweeps 1 --dump-sweep 0
                  --dav 1e-6 --with-data 0
  heff_syn24_su2_M1000_mid.npz: n=24 N=24 SU(2) M=1000, sweep 2 middle site
      ref_harness --ham syn_n24.FCIDUMP --M 1000 --sweeps 3 --dump-sweep 2
                  --noises 1e-5,1e-5,0 --dav 1e-6,1e-6,1e-7 --with-data 0
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from b2g.workloads import pack, unpack  # noqa: E402

DT = {"i4": np.int32, "u8": np.uint64, "f8": np.float64}


def read_dump(d):
    arrays, scalars = {}, {}
    with open(os.path.join(d, "manifest.txt")) as f:
        for ln in f:
            t = ln.split()
            if not t:
                continue
            if t[0].startswith("#"):
                scalars[t[0][1:]] = float(t[1])
            else:
                arrays[t[0]] = np.fromfile(os.path.join(d, t[0] + ".bin"), dtype=DT[t[1]], count=int(t[2]))
    return arrays, scalars


if __name__ == "__main__":
    a, s = read_dump(sys.argv[1])
    np.savez_compressed(sys.argv[2], **pack(a, s, sys.argv[3] if len(sys.argv) > 3 else ""))
    pairs, meta = unpack(np.load(sys.argv[2]))
    for k, v in pairs.items():
        assert np.array_equal(np.asarray(v).astype(np.float64), a[k].astype(np.float64)), k
    print(sys.argv[2], os.path.getsize(sys.argv[2]), "bytes;", meta)
