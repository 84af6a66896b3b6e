"""Runs block2's DMRG::solve with the GB300 drop-in (lib/dmrg_sweep) and
reads back what it reports.

The sweep program is block2's own two-site DMRG driven through its C++ API
(shim/dmrg_sweep.cpp); the GPU arms install shim/b2g_block2.hpp's
GpuTensorFunctions / GpuDMRG, so every Davidson solve runs on the device
while block2's environment, truncation and sweep logic run unchanged on the
host.  ``run_sweep`` builds the command line, runs it, and returns the JSON
the program writes plus, per stage, the per-site lines block2 prints at
iprint 2 (``Iteration`` output, src/dmrg/sweep_algorithm.hpp:151-166).
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import tempfile

from .integrals import hubbard_integrals, synthetic_integrals, write_fcidump  # noqa: F401

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SWEEP_BIN = os.path.join(PKG, "lib", "dmrg_sweep")

_SITE = re.compile(r"--> Site =\s*(\d+)-\s*(\d+) \.\. Mmps =\s*(\d+) Ndav =\s*(\d+) E =\s*(\S+) "
                   r"Error =\s*(\S+) FLOPS =\s*(\S+) Tdav =\s*(\S+) T =\s*(\S+)")
_SWEEP = re.compile(r"Sweep =\s*(\d+) \| Direction =\s*(\w+)")
_STAGE = re.compile(r"== stage (\S+):")


def parse_sites(stdout: str) -> dict:
    """Per stage tag, the per-site Davidson records block2 printed:
    (sweep, site, mmps, ndav, energy, error, mnk/s, tdav, t)."""
    out, tag, sweep = {}, None, -1
    for line in stdout.splitlines():
        m = _STAGE.search(line)
        if m:
            tag, sweep = m.group(1), -1
            out[tag] = []
            continue
        m = _SWEEP.search(line)
        if m:
            sweep = int(m.group(1))
            continue
        m = _SITE.search(line)
        if m and tag is not None:
            out[tag].append({"sweep": sweep, "site": int(m.group(1)), "mmps": int(m.group(3)),
                             "ndav": int(m.group(4)), "energy": float(m.group(5)),
                             "error": float(m.group(6)), "mnk_per_s": float(m.group(7)),
                             "tdav": float(m.group(8)), "t": float(m.group(9))})
    return out


def fcidump_synthetic(path: str, n: int, seed: int = 0) -> str:
    """Writes the synthetic ab initio Hamiltonian of n orbitals (n electrons)."""
    h, eri, ecore = synthetic_integrals(n, seed)
    write_fcidump(path, h, eri, ecore, nelec=n, ms2=0)
    return path


def run_sweep(*, binary: str = SWEEP_BIN, ham: str = "hubbard", L: int = 16, U: float = 4.0,
              t: float = 1.0, sym: str = "su2", M=(250,), sweeps: int = 4, noises=(0.0,),
              dav=(1e-10,), arms=("gpu:fp64",), warm_sweeps: int = 0, warm_M=None,
              warm_noises=None, warm_dav=None, warm_device: str = "cpu", threads: int | None = None,
              seed: int = 1234, start_site: int = 0, end_site: int = -1, workdir: str | None = None,
              timeout: float | None = None, env: dict | None = None, dump_heff: str | None = None,
              dump_arm: int = 0, dump_sweep: int = -1, dump_site: int = -1, nroots: int = 1,
              stack_gb: float = 4.0, noise_type: str = "dm", noise_on_device: bool = True,
              pdm: int = 0, pdm_order: int = 1) -> dict:
    """Runs one dmrg_sweep invocation and returns its JSON report with
    ``sites`` (parse_sites of its output), ``stdout`` and ``cmd``.  With
    dump_heff, GPU arm ``dump_arm`` writes the H_eff of ``dump_site`` (default:
    the middle site) in its sweep ``dump_sweep`` to that directory
    (b2g.problem.load_dump reads it).  stack_gb sizes block2's DataFrame stack
    (4 GB is enough up to M = 1000; n = 32 M = 2000 needs more).  noise_type "dm"
    is block2's NoiseTypes::DensityMatrix, "perturbative" its ReducedPerturbative,
    "perturbative-full" Perturbative, "perturbative-lowmem" ReducedPerturbativeLowMem and
    "perturbative-collected" ReducedPerturbativeCollected (pyblock2's driver default)
    (GPU arms run that product on the device unless noise_on_device is false).  pdm=1
    adds each arm's 1-PDM (block2's Expect on the arm's final MPS, on the arm's device:
    "pdm1"); pdm=2 also gives GPU arms block2's own 1-PDM of the same MPS ("pdm1_host").
    pdm_order=2 computes the 2-PDM instead (keys "pdm2", "pdm2_host", ...)."""
    if not os.path.exists(binary):
        raise FileNotFoundError(f"{binary} is not built (build() needs block2's headers)")
    lst = lambda v: ",".join(str(x) for x in v)  # noqa: E731
    threads = threads or len(os.sched_getaffinity(0))
    own = workdir is None
    wd = tempfile.mkdtemp(prefix="b2g_sweep_") if own else os.path.abspath(workdir)
    os.makedirs(wd, exist_ok=True)
    js = os.path.join(wd, "result.json")
    cmd = [binary, "--ham", ham, "--L", str(L), "--U", str(U), "--t", str(t), "--sym", sym,
           "--M", lst(M), "--sweeps", str(sweeps), "--noises", lst(noises), "--dav", lst(dav),
           "--arms", ",".join(arms), "--threads", str(threads), "--seed", str(seed),
           "--iprint", "2", "--json", js, "--scratch", os.path.join(wd, "scratch"),
           "--start-site", str(start_site), "--end-site", str(end_site), "--nroots", str(nroots),
           "--stack-gb", str(stack_gb), "--noise-type", noise_type,
           "--noise-on-device", "1" if noise_on_device else "0", "--pdm", str(int(pdm)),
           "--pdm-order", str(int(pdm_order))]
    if dump_heff:
        cmd += ["--dump-heff", os.path.abspath(dump_heff), "--dump-arm", str(dump_arm),
                "--dump-sweep", str(dump_sweep), "--dump-site", str(dump_site)]
    if warm_sweeps:
        cmd += ["--warm-sweeps", str(warm_sweeps), "--warm-M", lst(warm_M or M),
                "--warm-noises", lst(warm_noises or noises), "--warm-dav", lst(warm_dav or dav),
                "--warm-device", warm_device]
    e = dict(os.environ)
    e.setdefault("OPENBLAS_NUM_THREADS", "1")
    e["OMP_NUM_THREADS"] = str(threads)
    if env:
        e.update(env)
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, env=e, cwd=wd)
    if r.returncode != 0:
        raise RuntimeError(f"dmrg_sweep failed ({r.returncode}):\n{r.stdout[-4000:]}\n{r.stderr[-4000:]}")
    with open(js) as f:
        res = json.load(f)
    res["sites"] = parse_sites(r.stdout)
    res["stdout"] = r.stdout
    res["cmd"] = cmd
    if own:
        import shutil
        shutil.rmtree(wd, ignore_errors=True)
    return res
