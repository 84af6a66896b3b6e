"""Differentiation form at the n=16 M=500 configuration: integral derivatives of
the converged DMRG energy from the adjoint of H_eff*psi, against the
reference's own 1-/2-PDM and against central finite differences.

The reference (oracle/_ref/ref_harness, block2's own CPU DMRG) converges the
synthetic ab initio Hamiltonian n=16, N=16, S=0, SU(2) at M=500 (8 sweeps),
computes the spin-summed 1-/2-PDM of the final MPS with its Expect sweep, and
for every listed FCIDUMP rebuilds the H_eff of the middle site (sites 7-8) at
that same fixed MPS.  The listed FCIDUMPs are the base Hamiltonian and, for 20
seeded random directions D_k in integral space (a symmetric one-electron part
and an eight-fold-symmetric two-electron part), the Hamiltonians at
theta +- t D_k with t = 1e-5.  At a fixed MPS the energy is linear in the
integrals, E(theta) = <psi|H_eff(ops(theta))|psi> + E_core, and by
Hellmann-Feynman its derivative is the converged energy's.  Per direction:

  * pdm  = sum_ij h_D[i,j] dm1[i,j] + 1/2 sum_ijkl (ij|kl)_D dm2[i,k,l,j]
           (the reference's PDMs; the convention is pinned by the energy
           identity E = sum h dm1 + 1/2 sum (ij|kl) dm2[i,k,l,j] + E_core);
  * fd   = (E(theta + t D) - E(theta - t D)) / (2 t), each E the Rayleigh
           quotient of the centre tensor with the reference's H_eff replayed
           by the oracle;
  * adj  = <dE/dops, (ops(theta + t D) - ops(theta - t D)) / (2 t)> with
           dE/dops from the adjoint -- the oracle's numpy adjoint here, and,
           with --gpu, the library's adjoint kernel behind torch.autograd
           (b2g.autodiff.heff_apply) on cuda:0.

The summary (a few KB, no operator data) is written to
tests/golden/syn16_M500_grad.json; the dumps (about 22 GB) stay in
tests/golden/_raw/grad16 unless --no-keep is given.  Test infrastructure: runs the
reference; nothing of the product imports it.

    python tests/golden/make_grad_syn16.py [--threads 8] [--gpu] [--reuse]
    python tests/golden/make_grad_syn16.py --gpu-check DUMP_DIR OUT.json   # GPU machine, copied dumps
    python tests/golden/make_grad_syn16.py --gpu-vs-oracle DUMP OUT.json    # GPU machine, a drop-in dump
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from b2g.integrals import synthetic_integrals, write_fcidump  # noqa: E402
from b2g.problem import PAIR_FIELDS  # noqa: E402
from make_fixtures import HARNESS, RAW, read_dump  # noqa: E402

N, M, T, NDIR = 16, 500, 1e-5, 20
SITE = N // 2 - 1
ARGS = ["--M", str(M), "--sym", "su2", "--sweeps", "8", "--seed", "1234", "--dav", "1e-12",
        "--dump-sweep", "99", "--pdm", "1", "--perturb-site", str(SITE), "--perturb-threads", "1"]
OUT_JSON = os.path.join(HERE, "syn16_M500_grad.json")
NPROJ = 8   # seeded random projections of dE/dops (the GPU check compares these)


def projection(k: int, size: int) -> np.ndarray:
    return np.random.default_rng(9000 + k).standard_normal(size)


def site_dump(out: str, k: int):
    d = os.path.join(out, f"perturb{k}")
    (sd,) = [x for x in os.listdir(d) if x.startswith("sweep")]
    return read_dump(os.path.join(d, sd))


def gpu_gradient(base_a: dict, base_s: dict):
    """dE/dops = d<psi|H_eff(ops)|psi>/d ops at the normalised centre tensor,
    by the library's adjoint kernel behind torch.autograd on cuda:0."""
    from b2g.capi import PairSeq
    return gpu_gradient_of(PairSeq({k: base_a[k] for k in PAIR_FIELDS}), base_a["ops"], base_a["psi"],
                           int(base_s["psi_size"]), int(base_s["sigma_size"]))


def gpu_gradient_of(seq, ops, psi, psi_size: int, sigma_size: int):
    import torch

    import b2g
    from b2g.autodiff import heff_apply
    psi = np.array(psi, dtype=np.float64)
    psi_n = psi / np.linalg.norm(psi)
    ctx = b2g.Context(0)
    h = b2g.EffectiveHamiltonian(ctx, seq, ops, psi_size, sigma_size)
    ops_t = torch.from_numpy(np.array(ops)).to("cuda:0").requires_grad_(True)
    x = torch.from_numpy(psi_n).to("cuda:0")
    f = torch.dot(x, heff_apply(h, ops_t, x))
    f.backward()   # warm-up (adjoint schedule built on first use)
    ops_t.grad = None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    f = torch.dot(x, heff_apply(h, ops_t, x))
    f.backward()
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    g = ops_t.grad.cpu().numpy()
    h.close()
    ctx.close()
    return g, t


def gpu_vs_oracle(dump_dir: str, out_path: str):
    """On a GPU machine: at an H_eff the drop-in dumped during a sweep
    (b2g.problem.load_dump; e.g. bench.py --workload syn16 --keep-dump DIR),
    dE/dops from the library's adjoint kernel against the oracle's numpy
    adjoint, elementwise (the derivative the integral chain above uses)."""
    from oracle import oracle

    from b2g.problem import load_dump
    prob = load_dump(dump_dir)
    psi = np.array(prob.extra.get("psi_converged", prob.psi), dtype=np.float64)
    g, t = gpu_gradient_of(prob.seq(), prob.ops, psi, prob.psi_size, prob.sigma_size)
    psi_n = psi / np.linalg.norm(psi)
    t0 = time.perf_counter()
    gc, _ = oracle.adjoint(prob.seq(), prob.ops, psi_n, psi_n)
    tc = time.perf_counter() - t0
    res = {"site": int(prob.meta["site"]), "sweep": int(prob.meta["isweep"]), "n_pairs": int(prob.seq().n),
           "ops_size": int(prob.ops.size), "rel_diff_norm": float(np.linalg.norm(g - gc) / np.linalg.norm(gc)),
           "max_abs_diff_over_max": float(np.abs(g - gc).max() / np.abs(gc).max()),
           "seconds_gpu_forward_backward": t, "seconds_oracle_adjoint": tc}
    with open(out_path, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res), flush=True)


def gpu_check(dump_dir: str, out_path: str):
    """On a GPU machine: the library's adjoint at the dumped base site against
    the oracle adjoint's seeded projections stored in the summary."""
    with open(OUT_JSON) as f:
        summ = json.load(f)
    base_a, base_s = site_dump(dump_dir, 0)
    g, t = gpu_gradient(base_a, base_s)
    proj = [float(g @ projection(k, g.size)) for k in range(NPROJ)]
    cpu = summ["adjoint_projections"]["cpu"]
    res = {"gpu": proj, "cpu": cpu, "grad_norm_gpu": float(np.linalg.norm(g)),
           "grad_norm_cpu": summ["adjoint_projections"]["grad_norm_cpu"],
           "max_rel_diff": max(abs(a - b) / max(abs(b), 1e-300) for a, b in zip(proj, cpu)),
           "seconds_forward_backward": t}
    with open(out_path, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res), flush=True)


def direction(k: int):
    """Seeded random direction in integral space: symmetric h_D, 8-fold symmetric
    eri_D, scaled so that its largest element is 1 (each integral moves by at
    most t): the energy at fixed MPS is linear in the integrals, so the central
    difference has no truncation error and a larger signal only lowers its
    rounding error (unit-norm directions move each integral by ~1e-7 t and
    leave the differences of two 87 Ha energies at the 1e-6 relative level)."""
    rng = np.random.default_rng(7000 + k)
    h = rng.standard_normal((N, N))
    h = 0.5 * (h + h.T)
    x = rng.standard_normal((N, N, N, N))
    e = (x + x.transpose(1, 0, 2, 3) + x.transpose(0, 1, 3, 2) + x.transpose(1, 0, 3, 2)
         + x.transpose(2, 3, 0, 1) + x.transpose(3, 2, 0, 1) + x.transpose(2, 3, 1, 0)
         + x.transpose(3, 2, 1, 0)) / 8.0
    s = 1.0 / max(np.abs(h).max(), np.abs(e).max())
    return h * s, e * s


def base_layout_map(base: dict, other: dict) -> np.ndarray:
    """Index map idx such that other["ops"][idx] is the other run's operator
    data in the base run's blob layout.  The harness packs operator matrices
    in address order, which can differ between runs, while the pair sequence
    (order, shapes, coefficients) is the same: pair i references the same
    operator block in both, at base offset b0[i] / a1[i] and other offset
    b0[i] / a1[i].  Every referenced block is mapped; the map must be one to one."""
    starts, lens, dsts = [], [], []
    for off_k, tr_k, r_k, c_k, ld_k in (("b0", "tb0", "k0", "n0", "ldb0"), ("a1", "ta1", "m1", "k1", "lda1")):
        tr = base[tr_k].astype(bool)
        rows, cols, ld = base[r_k].astype(np.int64), base[c_k].astype(np.int64), base[ld_k].astype(np.int64)
        ext = np.where(tr, (cols - 1) * ld + rows, (rows - 1) * ld + cols)
        ext = np.where((rows > 0) & (cols > 0), ext, 0)
        dsts.append(base[off_k].astype(np.int64))
        starts.append(other[off_k].astype(np.int64))
        lens.append(ext)
    dst, src, ln = np.concatenate(dsts), np.concatenate(starts), np.concatenate(lens)
    key = np.unique(np.stack([dst, src, ln], 1), axis=0)
    if np.unique(key[:, 0]).size != key.shape[0]:
        raise RuntimeError("a base operator block maps to two blocks of the other run")
    idx = np.arange(base["ops"].size, dtype=np.int64)
    for d, s_, n in key:
        idx[d:d + n] = np.arange(s_, s_ + n)
    return idx


def rayleigh(seq, ops, psi, nsig, oracle) -> float:
    sig = oracle.replay(seq, ops, psi, nsig)
    return float(psi @ sig / (psi @ psi))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--gpu", action="store_true", help="also the library's adjoint kernel on cuda:0")
    ap.add_argument("--reuse", action="store_true", help="reuse an existing harness run in _raw/grad16")
    ap.add_argument("--no-keep", action="store_true", help="delete the dumps afterwards")
    ap.add_argument("--gpu-check", nargs=2, metavar=("DUMP_DIR", "OUT_JSON"),
                    help="only compare the library's adjoint at DUMP_DIR's base site with the stored "
                         "oracle projections (a GPU machine with a copy of the dumps)")
    ap.add_argument("--gpu-vs-oracle", nargs=2, metavar=("DUMP_DIR", "OUT_JSON"),
                    help="only compare the library's adjoint with the oracle's at an H_eff the drop-in "
                         "dumped (bench.py --keep-dump)")
    a = ap.parse_args()
    if a.gpu_vs_oracle:
        gpu_vs_oracle(*a.gpu_vs_oracle)
        return
    if a.gpu_check:
        gpu_check(*a.gpu_check)
        return
    from b2g.capi import PairSeq
    from oracle import oracle
    h0, eri0, ec = synthetic_integrals(N, seed=0)
    out = os.path.join(RAW, "grad16")
    dirs = [direction(k) for k in range(NDIR)]
    t_h = None
    if not (a.reuse and os.path.isdir(os.path.join(out, "pdm"))):
        if os.path.exists(out):
            shutil.rmtree(out)
        os.makedirs(out)
        dumps = [os.path.join(out, "base.FCIDUMP")]
        write_fcidump(dumps[0], h0, eri0, ec, nelec=N)
        for k, (hd, ed) in enumerate(dirs):
            for sgn, tag in ((+1, "p"), (-1, "m")):
                path = os.path.join(out, f"d{k:02d}{tag}.FCIDUMP")
                write_fcidump(path, h0 + sgn * T * hd, eri0 + sgn * T * ed, ec, nelec=N)
                dumps.append(path)
        if not os.path.exists(HARNESS):
            subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"),
                            os.environ.get("BLOCK2_SRC", ""), "harness"], check=True)
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
        cmd = [HARNESS, "--ham", dumps[0], *ARGS, "--perturb", ",".join(dumps), "--threads", str(a.threads),
               "--out", out]
        t0 = time.perf_counter()
        r = subprocess.run(cmd, capture_output=True, text=True, env=env)
        t_h = time.perf_counter() - t0
        with open(os.path.join(out, "log.txt"), "w") as f:
            f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    res_a, res_s = read_dump(os.path.join(out, "result"))
    pdm_a, _ = read_dump(os.path.join(out, "pdm"))
    dm1 = pdm_a["dm1"].reshape(N, N)
    dm2 = pdm_a["dm2"].reshape(N, N, N, N)

    def site(k):
        return site_dump(out, k)

    base_a, base_s = site(0)
    seq = PairSeq({k: base_a[k] for k in PAIR_FIELDS})
    nsig = int(base_s["sigma_size"])
    psi = np.array(base_a["psi"], dtype=np.float64)
    psi_n = psi / np.linalg.norm(psi)
    e_state = rayleigh(seq, base_a["ops"], psi, nsig, oracle) + ec
    e_pdm = float(np.einsum("ij,ij->", h0, dm1)) + 0.5 * float(np.einsum("ijkl,iklj->", eri0, dm2)) + ec
    print(f"E(MPS) = {e_state:.12f}, from the PDMs {e_pdm:.12f}, last sweep {float(res_s['energy']):.12f}",
          flush=True)
    t0 = time.perf_counter()
    g_cpu, _ = oracle.adjoint(seq, base_a["ops"], psi_n, psi_n)
    t_adj_cpu = time.perf_counter() - t0
    projections = [float(g_cpu @ projection(k, g_cpu.size)) for k in range(NPROJ)]
    g_gpu, t_adj_gpu = None, None
    if a.gpu:
        g_gpu, t_adj_gpu = gpu_gradient(base_a, base_s)
    rows = []
    for k, (hd, ed) in enumerate(dirs):
        (ap_, _), (am_, _) = site(1 + 2 * k), site(2 + 2 * k)
        for x_ in (ap_, am_):
            for f_ in PAIR_FIELDS:
                if f_ not in ("b0", "a1") and not np.array_equal(x_[f_], base_a[f_]):
                    raise RuntimeError(f"direction {k}: pair structure differs ({f_})")
        op_p = ap_["ops"][base_layout_map(base_a, ap_)]
        op_m = am_["ops"][base_layout_map(base_a, am_)]
        dops = (op_p - op_m) / (2 * T)
        pdm = float(np.sum(hd * dm1)) + 0.5 * float(np.einsum("ijkl,iklj->", ed, dm2))
        fd = (rayleigh(seq, op_p, psi, nsig, oracle) - rayleigh(seq, op_m, psi, nsig, oracle)) / (2 * T)
        row = {"direction": k, "pdm": pdm, "fd": fd, "adjoint_cpu": float(g_cpu @ dops)}
        if g_gpu is not None:
            row["adjoint_gpu"] = float(g_gpu @ dops)
        rows.append(row)
        print(row, flush=True)

    def rel(key, ref):
        return max(abs(r[key] - r[ref]) / max(abs(r[ref]), 1e-300) for r in rows)

    summary = {
        "what": ("integral derivatives of the converged energy, n=16 N=16 S=0 SU(2) M=500, middle site "
                 f"{SITE}-{SITE + 1} of the reference's converged MPS; {NDIR} seeded random integral "
                 f"directions, central step {T}"),
        "energy_mps": e_state, "energy_from_pdms": e_pdm, "last_sweep_energy": float(res_s["energy"]),
        "n_pairs": int(seq.n), "ops_size": int(base_a["ops"].size), "psi_size": int(psi.size),
        "rows": rows,
        "max_rel_err": {"adjoint_cpu_vs_pdm": rel("adjoint_cpu", "pdm"), "fd_vs_pdm": rel("fd", "pdm"),
                        "adjoint_cpu_vs_fd": rel("adjoint_cpu", "fd")},
        "bound": 1e-6, "seconds": {"harness": t_h, "adjoint_cpu": t_adj_cpu, "adjoint_gpu": t_adj_gpu},
        "adjoint_projections": {"seeds": [9000 + k for k in range(NPROJ)], "cpu": projections,
                                "grad_norm_cpu": float(np.linalg.norm(g_cpu))},
    }
    if g_gpu is not None:
        summary["max_rel_err"]["adjoint_gpu_vs_pdm"] = rel("adjoint_gpu", "pdm")
        summary["max_rel_err"]["adjoint_gpu_vs_fd"] = rel("adjoint_gpu", "fd")
        summary["gpu_vs_cpu_adjoint_rel"] = float(np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu))
    with open(OUT_JSON, "w") as f:
        json.dump(summary, f, indent=1)
    print(json.dumps(summary["max_rel_err"]), flush=True)
    if a.no_keep:
        shutil.rmtree(out, ignore_errors=True)


if __name__ == "__main__":
    main()
