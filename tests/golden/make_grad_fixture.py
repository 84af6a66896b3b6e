"""Generates tests/golden/syn8_su2_s0_grad.npz: integral derivatives of a site
energy, computed by the reference itself, for the differentiation form.

The first site of the first sweep (sweep 0, sites 0-1) is the one place where
the effective Hamiltonian depends on the integrals only through the MPO: its
environments are built from the seeded random initial MPS
(MPS::random_canonicalize), which does not see the Hamiltonian.  There the
operator blob is a linear function of the integrals, and the site energy
E(theta) = lowest eigenvalue of H_eff(ops(theta)).

For each integral parameter theta_k (a symmetric one-electron element h_pq, or
an eight-fold-symmetric two-electron element (pq|rs)), the reference harness
(oracle/_ref/ref_harness, the reference's own CPU DMRG) is run at
theta_k +- delta.  Stored per parameter:
  * jac_k = (ops(+delta) - ops(-delta)) / (2 delta), sparse -- the integral ->
    operator Jacobian column of the reference's MPO/environment construction
    (exact: the blob is linear in the integrals at fixed MPS);
  * e_plus_k, e_minus_k -- the reference's own converged site energies.
The check (tests/test_adjoint.py): dE/dtheta_k = <dE/dops, jac_k> with dE/dops
from the adjoint kernel (Hellmann-Feynman) equals the reference's central
difference (e_plus_k - e_minus_k) / (2 delta).

A second fixture, syn8_su2_conv_grad.npz, does the same at the converged MPS
of a full run and pins the derivatives to the reference's own 1-/2-PDM
(converged(), below); a third, syn8_su2_conv_fullgrad.npz, holds the Jacobian
for every independent integral there (full_gradient()).

Usage (needs the reference harness; not run on GPU machines):
    python tests/golden/make_grad_fixture.py
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
sys.path.insert(0, HERE)

from b2g.integrals import synthetic_integrals, write_fcidump  # noqa: E402
from b2g.problem import PAIR_FIELDS  # noqa: E402
from make_fixtures import HARNESS, RAW, read_dump  # noqa: E402

N = 8
DELTA = 1e-4
ARGS = ["--M", "60", "--sym", "su2", "--sweeps", "1", "--dump-sweep", "0", "--dump-site", "0", "--seed", "1234",
        "--dav", "1e-16"]
H_PARAMS = [(0, 0), (3, 3), (7, 7), (0, 1), (2, 5), (1, 6)]
ERI_PARAMS = [(0, 0, 0, 0), (0, 0, 1, 1), (0, 1, 0, 1), (1, 2, 3, 4)]


def eri_orbit(p, q, r, s):
    return {(p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
            (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)}


def block_extent(trans, rows, cols, ld):
    """Doubles spanned by a stored block op(X) of shape rows x cols, leading dim ld."""
    return (cols - 1) * ld + rows if trans else (rows - 1) * ld + cols


def to_base_layout(base, other):
    """The operator values of another run, moved into the base run's blob layout.

    The harness packs operator matrices in address order, which can change
    between runs; the pair sequence itself (order, shapes, coefficients) does
    not.  Pair i references the same operator block in both runs, so the
    block at base offset b0[i] (a1[i]) holds other["ops"] at other's b0[i]
    (a1[i]).  Every referenced block is moved; the mapping must be one to one."""
    out = np.array(base["ops"], copy=True)
    seen = {}
    for off_k, tr_k, r_k, c_k, ld_k in (("b0", "tb0", "k0", "n0", "ldb0"), ("a1", "ta1", "m1", "k1", "lda1")):
        for i in range(base[off_k].size):
            x, y = int(base[off_k][i]), int(other[off_k][i])
            e = block_extent(int(base[tr_k][i]), int(base[r_k][i]), int(base[c_k][i]), int(base[ld_k][i]))
            if seen.setdefault(x, (y, e)) != (y, e):
                raise RuntimeError("operator block mapping between runs is not one to one")
            out[x:x + e] = other["ops"][y:y + e]
    return out


def run(tag, h, eri, ec):
    out = os.path.join(RAW, "grad", tag)
    if os.path.exists(out):
        shutil.rmtree(out)
    os.makedirs(out)
    fcidump = os.path.join(out, "FCIDUMP")
    write_fcidump(fcidump, h, eri, ec, nelec=N)
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    cmd = [HARNESS, "--ham", fcidump, *ARGS, "--threads", "1", "--out", out]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"{tag}: harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    site = os.path.join(out, "sweep0_site0")
    pre_a, pre_s = read_dump(site)
    post_a, post_s = read_dump(os.path.join(site, "post"))
    return pre_a, pre_s, post_a, post_s


def perturbed(h0, eri0, kind, idx, sgn):
    h, eri = h0.copy(), eri0.copy()
    if kind == "h":
        p, q = idx
        h[p, q] += sgn * DELTA
        if p != q:
            h[q, p] += sgn * DELTA
    else:
        for t in eri_orbit(*idx):
            eri[t] += sgn * DELTA
    return h, eri


def first_site():
    h0, eri0, ec = synthetic_integrals(N, seed=0)
    base_a, base_s, base_post, base_post_s = run("base", h0, eri0, ec)
    labels, jac_idx, jac_val, jac_ptr, e_plus, e_minus = [], [], [], [0], [], []
    params = [("h", p) for p in H_PARAMS] + [("eri", p) for p in ERI_PARAMS]
    lin_worst = 0.0
    for kind, idx in params:
        runs = []
        for sgn in (+1, -1):
            h, eri = perturbed(h0, eri0, kind, idx, sgn)
            tag = f"{kind}_{'_'.join(map(str, idx))}_{'p' if sgn > 0 else 'm'}"
            a, s, pa, ps = run(tag, h, eri, ec)
            for k in PAIR_FIELDS:
                if k not in ("b0", "a1") and not np.array_equal(a[k], base_a[k]):
                    raise RuntimeError(f"{tag}: pair structure differs from the base run ({k})")
            runs.append((to_base_layout(base_a, a), ps["energy"]))
        (op_p, e_p), (op_m, e_m) = runs
        d = (op_p - op_m) / (2 * DELTA)
        # the blob is linear in the integrals: both one-sided differences agree
        base_ops = to_base_layout(base_a, base_a)
        lin = np.linalg.norm((op_p - base_ops) - (base_ops - op_m)) / max(
            np.linalg.norm(op_p - op_m), 1e-300)
        lin_worst = max(lin_worst, lin)
        nz = np.nonzero(np.abs(d) > 1e-9 * np.abs(d).max())[0]
        labels.append(f"{kind}{list(idx)}")
        jac_idx.append(nz.astype(np.int64))
        jac_val.append(d[nz])
        jac_ptr.append(jac_ptr[-1] + nz.size)
        e_plus.append(e_p)
        e_minus.append(e_m)
        print(f"{labels[-1]}: jac nnz={nz.size} dE/dtheta(ref FD)={(e_p - e_m) / (2 * DELTA):.10f} "
              f"linearity {lin:.1e}")
    meta = {"name": "syn8_su2_s0_grad", "kind": "integral_gradient",
            "description": "synthetic ab initio n=8 N=8 (seed 0), SU(2), M=60, sweep 0 sites 0-1: "
                           "integral -> operator Jacobian columns and the reference's site energies "
                           "at theta +- delta",
            "harness_args": ARGS, "delta": DELTA, "labels": labels,
            "energy": base_post_s["energy"], "conv_thrd": base_s["conv_thrd"],
            "linearity_worst": lin_worst,
            "param_convention": "h[p,q]: h_pq and h_qp move together (one symmetric element); "
                                "eri[p,q,r,s]: all eight symmetry-equivalent entries move together"}
    path = os.path.join(HERE, "syn8_su2_s0_grad.npz")
    np.savez_compressed(
        path, **{k: base_a[k] for k in PAIR_FIELDS}, ops=base_a["ops"], psi=base_a["psi"],
        psi_final=base_post["psi"], psi_size=np.int64(base_s["psi_size"]),
        sigma_size=np.int64(base_s["sigma_size"]),
        jac_idx=np.concatenate(jac_idx), jac_val=np.concatenate(jac_val),
        jac_ptr=np.array(jac_ptr, dtype=np.int64), e_plus=np.array(e_plus), e_minus=np.array(e_minus),
        meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8))
    print(f"-> {path} ({os.path.getsize(path)} bytes), base E={meta['energy']:.12f}, "
          f"linearity worst {lin_worst:.1e}")


CONV_ARGS = ["--M", "60", "--sym", "su2", "--sweeps", "8", "--seed", "1234", "--dav", "1e-14",
             "--dump-sweep", "99", "--pdm", "1", "--perturb-site", "3"]


def converged():
    """syn8_su2_conv_grad.npz: at the converged MPS of an 8-sweep run, the
    reference's 1-/2-PDM (Expect) and, for each parameter, the H_eff of the
    middle site (sites 3-4) built with the perturbed integrals at that same
    (fixed) MPS -- the harness walks the canonical centre there with a sweep
    whose Davidson keeps its initial guess.  The
    energy derivative at fixed MPS is <Psi|dH/dtheta|Psi>, i.e. the PDM
    element; the chain adjoint x Jacobian must reproduce it."""
    h0, eri0, ec = synthetic_integrals(N, seed=0)
    out = os.path.join(RAW, "grad", "conv")
    if os.path.exists(out):
        shutil.rmtree(out)
    os.makedirs(out)
    params = [("h", p) for p in H_PARAMS] + [("eri", p) for p in ERI_PARAMS]
    dumps = [os.path.join(out, "base.FCIDUMP")]
    write_fcidump(dumps[0], h0, eri0, ec, nelec=N)
    for kind, idx in params:
        for sgn in (+1, -1):
            h, eri = perturbed(h0, eri0, kind, idx, sgn)
            path = os.path.join(out, f"{kind}_{'_'.join(map(str, idx))}_{'p' if sgn > 0 else 'm'}.FCIDUMP")
            write_fcidump(path, h, eri, ec, nelec=N)
            dumps.append(path)
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    cmd = [HARNESS, "--ham", dumps[0], *CONV_ARGS, "--perturb", ",".join(dumps), "--threads", "1",
           "--out", out]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    res_a, res_s = read_dump(os.path.join(out, "result"))
    pdm_a, _ = read_dump(os.path.join(out, "pdm"))
    dm1 = pdm_a["dm1"].reshape(N, N)
    dm2 = pdm_a["dm2"].reshape(N, N, N, N)

    def site(k):
        d = os.path.join(out, f"perturb{k}")
        (sd,) = [x for x in os.listdir(d) if x.startswith("sweep")]
        return read_dump(os.path.join(d, sd))

    base_a, base_s = site(0)
    # the energy of the fixed MPS: the Rayleigh quotient of its centre tensor
    # with the centre's H_eff (the reference's replay, restated by the oracle)
    sys.path.insert(0, ROOT)
    from b2g.capi import PairSeq
    from oracle import oracle
    psi = base_a["psi"]
    sig = oracle.replay(PairSeq({k: base_a[k] for k in PAIR_FIELDS}), base_a["ops"], psi,
                        int(base_s["sigma_size"]))
    e_state = float(psi @ sig / (psi @ psi)) + ec
    # energy identity fixes the 2-PDM convention: E = sum h dm1 + 1/2 sum (ij|kl) dm2[i,k,l,j]
    e1 = float(np.einsum("ij,ij->", h0, dm1))
    e2 = 0.5 * float(np.einsum("ijkl,iklj->", eri0, dm2))
    print(f"E(MPS)={e_state:.12f}  sum h dm1 + 1/2 sum v dm2 = {e1 + e2 + ec:.12f} "
          f"(last sweep energy {float(res_s['energy']):.12f})")
    if abs(e1 + e2 + ec - e_state) > 1e-10:
        raise RuntimeError("PDM energy identity does not hold with the assumed convention")
    e_final = e_state
    labels, jac_idx, jac_val, jac_ptr, expect = [], [], [], [0], []
    lin_worst = 0.0
    base_ops = to_base_layout(base_a, base_a)
    for i, (kind, idx) in enumerate(params):
        (ap, _), (am, _) = site(1 + 2 * i), site(2 + 2 * i)
        for a in (ap, am):
            for k in PAIR_FIELDS:
                if k not in ("b0", "a1") and not np.array_equal(a[k], base_a[k]):
                    raise RuntimeError(f"{kind}{idx}: pair structure differs ({k})")
        op_p, op_m = to_base_layout(base_a, ap), to_base_layout(base_a, am)
        d = (op_p - op_m) / (2 * DELTA)
        lin = np.linalg.norm((op_p - base_ops) - (base_ops - op_m)) / max(np.linalg.norm(op_p - op_m), 1e-300)
        lin_worst = max(lin_worst, lin)
        nz = np.nonzero(np.abs(d) > 1e-9 * np.abs(d).max())[0]
        if kind == "h":
            p, q = idx
            ex = dm1[p, q] + (dm1[q, p] if p != q else 0.0)
        else:
            ex = 0.5 * sum(dm2[i_, k_, l_, j_] for (i_, j_, k_, l_) in eri_orbit(*idx))
        labels.append(f"{kind}{list(idx)}")
        jac_idx.append(nz.astype(np.int64))
        jac_val.append(d[nz])
        jac_ptr.append(jac_ptr[-1] + nz.size)
        expect.append(ex)
        print(f"{labels[-1]}: jac nnz={nz.size} PDM derivative={ex:.12f} linearity {lin:.1e}")
    meta = {"name": "syn8_su2_conv_grad", "kind": "integral_gradient_pdm",
            "description": "synthetic ab initio n=8 N=8 (seed 0), SU(2), M=60, converged 8-sweep MPS "
                           "(harness seed 1234): H_eff of the middle site (3-4), integral -> operator Jacobian "
                           "at that fixed MPS, and the reference's 1-/2-PDM (Expect)",
            "harness_args": CONV_ARGS, "delta": DELTA, "labels": labels, "energy": e_final,
            "linearity_worst": lin_worst,
            "pdm_convention": "E = sum_ij h_ij dm1[i,j] + 1/2 sum_ijkl (ij|kl) dm2[i,k,l,j] + E_core "
                              "(spin-summed spatial PDMs of Expect::get_1pdm_spatial / get_2pdm_spatial)",
            "param_convention": "h[p,q]: h_pq and h_qp move together; eri[p,q,r,s]: all eight "
                                "symmetry-equivalent entries move together"}
    path = os.path.join(HERE, "syn8_su2_conv_grad.npz")
    np.savez_compressed(
        path, **{k: base_a[k] for k in PAIR_FIELDS}, ops=base_ops, psi=base_a["psi"],
        psi_size=np.int64(base_s["psi_size"]), sigma_size=np.int64(base_s["sigma_size"]),
        jac_idx=np.concatenate(jac_idx), jac_val=np.concatenate(jac_val),
        jac_ptr=np.array(jac_ptr, dtype=np.int64), pdm_derivative=np.array(expect), dm1=dm1, dm2=dm2,
        meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8))
    print(f"-> {path} ({os.path.getsize(path)} bytes), linearity worst {lin_worst:.1e}")


def unique_params(n):
    """Every independent integral: h_pq (p >= q) and (pq|rs) (p >= q, r >= s, pq >= rs)."""
    pairs = [(i, j) for i in range(n) for j in range(i + 1)]
    hs = [("h", p) for p in pairs]
    es = [("eri", pairs[a] + pairs[b]) for a in range(len(pairs)) for b in range(a + 1)]
    return hs + es


def full_gradient():
    """syn8_su2_conv_fullgrad.npz: the integral -> operator Jacobian of the
    middle-site H_eff at the converged MPS (the run of converged()) for every
    independent integral, by one-sided differences (the blob is linear in the
    integrals at fixed MPS), with the reference's full 1-/2-PDM."""
    h0, eri0, ec = synthetic_integrals(N, seed=0)
    out = os.path.join(RAW, "grad", "full")
    if os.path.exists(out):
        shutil.rmtree(out)
    os.makedirs(out)
    params = unique_params(N)
    dumps = [os.path.join(out, "base.FCIDUMP")]
    write_fcidump(dumps[0], h0, eri0, ec, nelec=N)
    for k, (kind, idx) in enumerate(params):
        h, eri = perturbed(h0, eri0, kind, idx, +1)
        dumps.append(os.path.join(out, f"p{k}.FCIDUMP"))
        write_fcidump(dumps[-1], h, eri, ec, nelec=N)
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1")
    cmd = [HARNESS, "--ham", dumps[0], *CONV_ARGS, "--perturb", ",".join(dumps), "--threads", "1",
           "--out", out]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError(f"harness failed\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    pdm_a, _ = read_dump(os.path.join(out, "pdm"))
    dm1 = pdm_a["dm1"].reshape(N, N)
    dm2 = pdm_a["dm2"].reshape(N, N, N, N)

    def site(k):
        d = os.path.join(out, f"perturb{k}")
        (sd,) = [x for x in os.listdir(d) if x.startswith("sweep")]
        return read_dump(os.path.join(d, sd))

    base_a, base_s = site(0)
    base_ops = to_base_layout(base_a, base_a)
    jac_idx, jac_val, jac_ptr, expect, labels = [], [], [0], [], []
    for k, (kind, idx) in enumerate(params):
        a, _ = site(k + 1)
        for key in PAIR_FIELDS:
            if key not in ("b0", "a1") and not np.array_equal(a[key], base_a[key]):
                raise RuntimeError(f"{kind}{idx}: pair structure differs ({key})")
        d = (to_base_layout(base_a, a) - base_ops) / DELTA
        nz = np.nonzero(np.abs(d) > 1e-9 * max(np.abs(d).max(), 1e-300))[0]
        jac_idx.append(nz.astype(np.int32))
        jac_val.append(d[nz])
        jac_ptr.append(jac_ptr[-1] + nz.size)
        if kind == "h":
            p, q = idx
            expect.append(dm1[p, q] + (dm1[q, p] if p != q else 0.0))
        else:
            expect.append(0.5 * sum(dm2[i_, k_, l_, j_] for (i_, j_, k_, l_) in eri_orbit(*idx)))
        labels.append(f"{kind}{list(idx)}")
    meta = {"name": "syn8_su2_conv_fullgrad", "kind": "integral_gradient_full",
            "description": "synthetic ab initio n=8 N=8 (seed 0), SU(2), M=60, converged 8-sweep MPS "
                           "(harness seed 1234): middle-site (3-4) H_eff and its integral -> operator "
                           "Jacobian for every independent integral (one-sided, step delta), with the "
                           "reference's 1-/2-PDM",
            "harness_args": CONV_ARGS, "delta": DELTA, "labels": labels,
            "pdm_convention": "E = sum_ij h_ij dm1[i,j] + 1/2 sum_ijkl (ij|kl) dm2[i,k,l,j] + E_core",
            "param_convention": "h[p,q] (p >= q): h_pq and h_qp move together; eri[p,q,r,s] "
                                "(p >= q, r >= s, pq >= rs): all eight symmetry-equivalent entries move together"}
    path = os.path.join(HERE, "syn8_su2_conv_fullgrad.npz")
    np.savez_compressed(
        path, **{k: base_a[k] for k in PAIR_FIELDS}, ops=base_ops, psi=base_a["psi"],
        psi_size=np.int64(base_s["psi_size"]), sigma_size=np.int64(base_s["sigma_size"]),
        jac_idx=np.concatenate(jac_idx), jac_val=np.concatenate(jac_val),
        jac_ptr=np.array(jac_ptr, dtype=np.int64), pdm_derivative=np.array(expect), dm1=dm1, dm2=dm2,
        meta=np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8))
    print(f"-> {path} ({os.path.getsize(path)} bytes), {len(params)} parameters, "
          f"{jac_ptr[-1]} Jacobian entries")


if __name__ == "__main__":
    first_site()
    converged()
    full_gradient()
