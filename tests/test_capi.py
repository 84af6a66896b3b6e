"""C-ABI library: loads, exports every symbol include/b2g.h declares, and the
host-side plan builder (no GPU needed) validates sequences and schedules them."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, fixture_ids
import b2g
from b2g import capi


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "b2g.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(b2g_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    syms = declared_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(L, s), s
        assert s in capi.SIGNATURES, s


def test_version_and_error_string():
    assert capi.lib().b2g_version() >= 1
    assert isinstance(capi.lib().b2g_last_error(), bytes)


@pytest.mark.parametrize("name", fixture_ids())
def test_plan_stats(problems, name):
    p = problems[name]
    st = b2g.plan_stats(p.seq(), p.ops.size, p.psi_size, p.sigma_size)
    assert st["n_pairs"] == p.meta["n_pairs"]
    assert st["mnk"] == pytest.approx(p.meta["mnk"], rel=1e-12)
    assert 0 < st["n_work"] <= st["n_pairs"]
    assert st["mnk_executed"] <= st["mnk"] * (1 + 1e-12)
    assert st["n_regions"] >= 1 and st["n_tiles"] >= st["n_regions"]


def _mutated(p, field, value, idx=0):
    arrays = {k: np.array(v, copy=True) for k, v in p.pairs.items()}
    arrays[field][idx] = value
    return b2g.PairSeq(arrays)


def test_plan_rejects_bad_sequences(problems):
    p = problems[sorted(problems)[0]]
    with pytest.raises(b2g.B2GError) as e:
        b2g.plan_stats(_mutated(p, "a0", p.psi_size), p.ops.size, p.psi_size, p.sigma_size)
    assert e.value.code == capi.B2G_ERR_ARG
    with pytest.raises(b2g.B2GError) as e:
        b2g.plan_stats(_mutated(p, "c1", p.sigma_size), p.ops.size, p.psi_size, p.sigma_size)
    assert e.value.code == capi.B2G_ERR_ARG
    with pytest.raises(b2g.B2GError) as e:
        b2g.plan_stats(_mutated(p, "b0", p.ops.size), p.ops.size, p.psi_size, p.sigma_size)
    assert e.value.code == capi.B2G_ERR_ARG
    k = int(p.pairs["k1"][0])
    with pytest.raises(b2g.B2GError) as e:
        b2g.plan_stats(_mutated(p, "k1", k + 1), p.ops.size, p.psi_size, p.sigma_size)
    assert e.value.code in (capi.B2G_ERR_UNSUPPORTED, capi.B2G_ERR_ARG)
    with pytest.raises(b2g.B2GError) as e:
        b2g.plan_stats(_mutated(p, "m0", -1), p.ops.size, p.psi_size, p.sigma_size)
    assert e.value.code == capi.B2G_ERR_ARG


def test_empty_sequence_is_valid():
    arrays = {k: np.zeros(0) for k in b2g.problem.PAIR_FIELDS}
    st = b2g.plan_stats(b2g.PairSeq(arrays), 0, 10, 10)
    assert st["n_pairs"] == 0 and st["n_tiles"] == 0


def test_context_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(b2g.B2GError):
        b2g.Context(0)


def test_plan_rejects_offsets_that_wrap(problems):
    """An offset near 2^64 must not wrap the range check round to a small sum."""
    p = problems[sorted(problems)[0]]
    for field in ("a0", "b0", "a1", "c1"):
        with pytest.raises(b2g.B2GError) as e:
            b2g.plan_stats(_mutated(p, field, np.uint64(2**64 - 1)), p.ops.size, p.psi_size, p.sigma_size)
        assert e.value.code == capi.B2G_ERR_ARG, field


def test_noalloc_validates_before_touching_the_device(problems):
    """b2g_heff_apply_noalloc checks every pair on the host before any CUDA
    call, so out-of-range and wrapping offsets are refused here without a GPU
    (the pointers are never dereferenced)."""
    import ctypes as C
    import torch
    if torch.cuda.is_available():
        pytest.skip("host-only check; the GPU suite covers the device path")
    p = problems[sorted(problems)[0]]
    fake = C.c_void_p(16)
    for field, value in (("a0", p.psi_size), ("c1", p.sigma_size), ("b0", np.uint64(2**64 - 8)),
                         ("a1", np.uint64(2**64 - 1))):
        seq = _mutated(p, field, value)
        rc = capi.lib().b2g_heff_apply_noalloc(C.byref(seq.c), fake, p.ops.size, fake, p.psi_size,
                                               fake, p.sigma_size, 1.0, None)
        assert rc == capi.B2G_ERR_ARG, field
        assert b"out of range" in capi.lib().b2g_last_error()
