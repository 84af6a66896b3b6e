"""Generates the golden fixtures in this directory from the reference itself.

Runs oracle/_ref/ref_harness (the reference's own CPU DMRG, compiled from the
reference sources by oracle/build_ref.sh) on small configurations, and
converts each dumped effective-Hamiltonian problem into a compressed .npz
(b2g.HeffProblem): the recorded GEMM-pair sequence, the operator blob, psi,
sigma = H_eff*psi from the reference's Tasked replay, diag(H_eff), and the
reference's converged Davidson eigenvector/energy at that site.

Usage (needs the reference sources; not run on GPU machines):
    python tests/golden/make_fixtures.py [--only NAME]
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))

from b2g.integrals import synthetic_integrals, write_fcidump  # noqa: E402
from b2g.problem import HeffProblem, PAIR_FIELDS  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
RAW = os.path.join(HERE, "_raw")

# name -> (harness arguments, description)
CASES = {
    "hub8_su2": (["--L", "8", "--U", "4", "--M", "40", "--sym", "su2", "--sweeps", "4",
                  "--dump-sweep", "0", "--dav", "1e-10,1e-10,1e-10,1e-10"],
                 "Hubbard L=8 t=1 U=4 OBC half filling, SU(2), M=40, sweep 0 middle site"),
    "hub8_sz": (["--L", "8", "--U", "4", "--M", "40", "--sym", "sz", "--sweeps", "4",
                 "--dump-sweep", "0", "--dav", "1e-10,1e-10,1e-10,1e-10"],
                "Hubbard L=8 t=1 U=4 OBC half filling, SZ, M=40, sweep 0 middle site"),
    "syn8_su2": (["--ham", "@syn8", "--M", "60", "--sym", "su2", "--sweeps", "4",
                  "--dump-sweep", "1", "--dav", "1e-10,1e-10,1e-10,1e-10"],
                 "synthetic ab initio n=8 N=8 (seed 0), SU(2), M=60, sweep 1 middle site"),
    "syn8_sz": (["--ham", "@syn8", "--M", "50", "--sym", "sz", "--sweeps", "2",
                 "--dump-sweep", "1", "--dav", "1e-9,1e-9"],
                "synthetic ab initio n=8 N=8 (seed 0), SZ, M=50, sweep 1 middle site"),
    "hub16_su2_M250": (["--L", "16", "--U", "4", "--M", "250", "--sym", "su2", "--sweeps", "4",
                        "--dump-sweep", "2", "--dav", "1e-10,1e-10,1e-10,1e-10"],
                       "Hubbard L=16 t=1 U=4 OBC half filling, SU(2), M=250, sweep 2 middle site "
                       "(the plain-FP64 Hubbard configuration's H_eff)"),
}

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


def fcidump_for(tag, workdir):
    n = int(tag[3:])
    path = os.path.join(workdir, f"syn_n{n}.FCIDUMP")
    h, eri, ec = synthetic_integrals(n, seed=0)
    write_fcidump(path, h, eri, ec, nelec=n)
    return path


def write_qn(name, site_dir):
    """NAME_qn.npz: the quantum-number bookkeeping of the two-site wavefunction
    (input StateInfos, the reference's tensor products, connection info and
    block list) from the harness's qn dump."""
    qa, qs = read_dump(os.path.join(site_dir, "qn"))
    qpath = os.path.join(HERE, name + "_qn.npz")
    np.savez_compressed(
        qpath, su2=np.int32(qs["su2"]), is_wfn=np.int32(qs["is_wfn"]),
        total_memory=np.int64(qs["total_memory"]), **qa,
        meta=np.array(json.dumps({"name": name + "_qn", "kind": "quanta",
                                  "description": "two-site wavefunction bookkeeping at the site of " + name})))
    print(f"{name}_qn: blocks={qa['wfn_q'].size} ll={qa['ll_q'].size} rr={qa['rr_q'].size} "
          f"-> {os.path.getsize(qpath)} bytes")


def run_case(name, args, desc, qn_only=False):
    out = os.path.join(RAW, name)
    if os.path.exists(out):
        shutil.rmtree(out)
    os.makedirs(out)
    args = list(args)
    for i, a in enumerate(args):
        if a.startswith("@syn"):
            args[i] = fcidump_for(a[1:], out)
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    cmd = [HARNESS, *args, "--threads", "8", "--out", out]
    log = subprocess.run(cmd, capture_output=True, text=True, env=env)
    with open(os.path.join(out, "log.txt"), "w") as f:
        f.write(" ".join(cmd) + "\n" + log.stdout + log.stderr)
    if log.returncode != 0:
        raise RuntimeError(f"{name}: harness failed\n{log.stdout[-2000:]}\n{log.stderr[-2000:]}")
    res_a, res_s = read_dump(os.path.join(out, "result"))
    site_dirs = [d for d in os.listdir(out) if d.startswith("sweep")]
    assert len(site_dirs) == 1, site_dirs
    write_qn(name, os.path.join(out, site_dirs[0]))
    if qn_only:
        return
    pre_a, pre_s = read_dump(os.path.join(out, site_dirs[0]))
    post_a, post_s = read_dump(os.path.join(out, site_dirs[0], "post"))
    pairs = {k: pre_a[k] for k in PAIR_FIELDS}
    meta = {
        "name": name, "description": desc, "harness_args": args,
        "n_pairs": int(pre_s["n_pairs"]), "mnk": pre_s["mnk"], "const_e": pre_s["const_e"],
        "isweep": int(pre_s["isweep"]), "site": int(pre_s["site"]), "n_sites": int(pre_s["n_sites"]),
        "conv_thrd": pre_s["conv_thrd"], "def_min": int(pre_s["def_min"]), "def_max": int(pre_s["def_max"]),
        "davidson_energy": post_s["energy"],
        "final_energy": res_s["energy"],
        "sweep_energies": [float(x) for x in res_a["sweep_energies"]],
        "discarded_weights": [float(x) for x in res_a["discarded_weights"]],
    }
    extra = {"psi_final": post_a["psi"], "psi_block_rows": pre_a["psi_block_rows"],
             "psi_block_cols": pre_a["psi_block_cols"], "psi_block_shift": pre_a["psi_block_shift"]}
    prob = HeffProblem(pairs=pairs, ops=pre_a["ops"], psi_size=int(pre_s["psi_size"]),
                       sigma_size=int(pre_s["sigma_size"]), psi=pre_a["psi"], sigma=pre_a["sigma"],
                       diag=pre_a["diag"], meta=meta, extra=extra)
    path = os.path.join(HERE, name + ".npz")
    prob.save(path)
    print(f"{name}: pairs={meta['n_pairs']} ops={prob.ops.size} psi={prob.psi_size} "
          f"E_dav={meta['davidson_energy']:.12f} E_final={meta['final_energy']:.12f} "
          f"-> {os.path.getsize(path)} bytes")
    # the operator rotation that followed this site (same pair format)
    rdir = os.path.join(out, site_dirs[0], "rotation")
    if os.path.isdir(rdir):
        ra, rs = read_dump(rdir)
        rmeta = {"name": name + "_rot", "kind": "rotation",
                 "description": "operator rotation after the site of " + name + " ("
                                + ("right" if rs["trans"] else "left") + "_rotate)",
                 "n_pairs": int(rs["n_pairs"]), "trans": int(rs["trans"])}
        rot = HeffProblem(pairs={k: ra[k] for k in PAIR_FIELDS}, ops=ra["ops"],
                          psi_size=int(rs["psi_size"]), sigma_size=int(rs["sigma_size"]),
                          psi=ra["psi"], sigma=ra["sigma"], meta=rmeta)
        rpath = os.path.join(HERE, name + "_rot.npz")
        rot.save(rpath)
        print(f"{name}_rot: pairs={rmeta['n_pairs']} in={rot.psi_size} out={rot.sigma_size} "
              f"-> {os.path.getsize(rpath)} bytes")
    # the environment blocking that followed this site (block-level records)
    bdir = os.path.join(out, site_dirs[0], "blocking")
    if os.path.isdir(bdir):
        ba, bs = read_dump(bdir)
        bpath = os.path.join(HERE, name + "_blk.npz")
        np.savez_compressed(
            bpath, right=np.int32(bs["right"]), tmp_size=np.int64(bs["tmp_size"]), **ba,
            meta=np.array(json.dumps({"name": name + "_blk", "kind": "blocking",
                                      "description": "environment blocking ("
                                      + ("right" if bs["right"] else "left")
                                      + "_contract) after the site of " + name})))
        print(f"{name}_blk: iadd={int(bs['n_iadd'])} kron={int(bs['n_kron'])} env={ba['env'].size} "
              f"site={ba['site'].size} out={ba['out'].size} -> {os.path.getsize(bpath)} bytes")
    # density matrix of the converged psi and the reference's truncation/split
    tdir = os.path.join(out, site_dirs[0], "truncation")
    if os.path.isdir(tdir):
        ta, ts = read_dump(tdir)
        tpath = os.path.join(HERE, name + "_dm.npz")
        np.savez_compressed(
            tpath, psi=post_a["psi"], trace_right=np.int32(ts["trace_right"]),
            bond_dim=np.int32(ts["bond_dim"]), cutoff=np.float64(ts["cutoff"]),
            error=np.float64(ts["error"]), **{k: v for k, v in ta.items()},
            meta=np.array(json.dumps({"name": name + "_dm", "kind": "truncation",
                                      "description": "density-matrix truncation after the site of "
                                                     + name})))
        print(f"{name}_dm: dm blocks={ta['dm_dim'].size} states={int(ta['dm_dim'].sum())} "
              f"M={int(ts['bond_dim'])} error={ts['error']:.3e} -> {os.path.getsize(tpath)} bytes")


def dm_fixture_from_dump(site_dir, name, desc):
    """A *_dm.npz fixture from an existing harness site dump (for the large
    truncation case, whose reference run takes ~25 minutes: the synthetic
    n=24 M=1000 SU(2) run of block2-preview_gb300/workloads/make_workload.py,
    sweep 2 middle site)."""
    ta, ts = read_dump(os.path.join(site_dir, "truncation"))
    post_a, _ = read_dump(os.path.join(site_dir, "post"))
    keep = {k: v for k, v in ta.items() if not k.startswith(("left_data", "right_data", "rho"))}
    tpath = os.path.join(HERE, name + "_dm.npz")
    np.savez_compressed(
        tpath, psi=post_a["psi"], trace_right=np.int32(ts["trace_right"]),
        bond_dim=np.int32(ts["bond_dim"]), cutoff=np.float64(ts["cutoff"]),
        error=np.float64(ts["error"]), **keep,
        meta=np.array(json.dumps({"name": name + "_dm", "kind": "truncation", "description": desc,
                                  "split_tensors": False})))
    print(f"{name}_dm: dm blocks={ta['dm_dim'].size} states={int(ta['dm_dim'].sum())} "
          f"-> {os.path.getsize(tpath)} bytes")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    ap.add_argument("--qn-only", action="store_true", help="write only the NAME_qn.npz fixtures")
    ap.add_argument("--dm-from-dump", nargs=2, metavar=("SITE_DIR", "NAME"), default=None,
                    help="write NAME_dm.npz (spectrum and discarded weight only) from a site dump")
    a = ap.parse_args()
    if a.dm_from_dump:
        dm_fixture_from_dump(a.dm_from_dump[0], a.dm_from_dump[1],
                             "density-matrix truncation, synthetic ab initio n=24 N=24 (seed 0), "
                             "SU(2), M=1000, sweep 2 middle site (spectrum and discarded weight)")
        return
    if not os.path.exists(HARNESS):
        # block2 sources: $BLOCK2_SRC, else the staged copy (shim/stage_block2.py)
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"),
                        os.environ.get("BLOCK2_SRC", ""), "harness"], check=True)
    for name, (args, desc) in CASES.items():
        if a.only and name != a.only:
            continue
        run_case(name, args, desc, qn_only=a.qn_only)


if __name__ == "__main__":
    main()
