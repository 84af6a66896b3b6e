"""The allocation-free H_eff*psi entry point, b2g_heff_apply_noalloc.

It serves callers that may not call cudaMalloc -- a program that gives the
GPU a fixed memory budget up front, or code running where an allocation would
synchronize the device or upset its memory accounting.  They own psi, sigma
and the operator blob on the device; the entry point keeps its work matrices
in a fixed-size array compiled into the library.

The test calls it through the C ABI twice in a row and checks each result
against the regular entry point (b2g_heff_apply), within the same 1e-12
relative tolerance the other H_eff*psi tests use.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import b2g  # noqa: E402
from b2g import capi  # noqa: E402

RTOL = 1e-12
CASES = ["hub8_su2", "syn8_su2", "syn8_sz", "hub16_su2_M250"]


def rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


@pytest.mark.parametrize("name", CASES)
def test_noalloc_matches_regular_entry_twice(problems, name):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    if name not in problems:
        pytest.skip(f"fixture {name} missing")
    p = problems[name]
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ctx = b2g.Context(0)
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    ops = torch.from_numpy(p.ops).to(dev)
    rng = np.random.default_rng(5)
    seq = p.seq()
    L = capi.lib()
    for call in range(2):
        x = torch.from_numpy(p.psi if call == 0 else rng.standard_normal(p.psi_size)).to(dev)
        want = torch.zeros(p.sigma_size, dtype=torch.float64, device=dev)
        h(x, want, 0.75)
        ctx.synchronize()
        got = torch.zeros(p.sigma_size, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev)
        rc = L.b2g_heff_apply_noalloc(C.byref(seq.c), ops.data_ptr(), p.ops.size, x.data_ptr(), p.psi_size,
                                      got.data_ptr(), p.sigma_size, 0.75, C.c_void_p(stream.cuda_stream))
        capi.check(rc)
        torch.cuda.synchronize(dev)
        assert rel(got, want) <= RTOL, (call, rel(got, want))
    h.close()
    ctx.close()


def test_noalloc_rejects_out_of_range_pairs(problems):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    p = problems["hub8_su2"]
    arrays = {k: np.array(v, copy=True) for k, v in p.pairs.items()}
    arrays["a0"][0] = p.psi_size
    seq = b2g.PairSeq(arrays)
    dev = torch.device("cuda", 0)
    ops = torch.from_numpy(p.ops).to(dev)
    x = torch.zeros(p.psi_size, dtype=torch.float64, device=dev)
    y = torch.zeros(p.sigma_size, dtype=torch.float64, device=dev)
    rc = capi.lib().b2g_heff_apply_noalloc(C.byref(seq.c), ops.data_ptr(), p.ops.size, x.data_ptr(),
                                           p.psi_size, y.data_ptr(), p.sigma_size, 1.0, None)
    assert rc == capi.B2G_ERR_ARG
