"""Environment blocking (left_contract / right_contract after a dumped site):
the reference's own block-level records replayed by the oracle (CPU) and by
b2g_block_contract (GPU), against the enlarged block's operators the
reference computed (fixtures *_blk.npz, tests/golden/make_fixtures.py)."""
from __future__ import annotations

import glob
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle  # noqa: E402

BLK = sorted(glob.glob(os.path.join(HERE, "golden", "*_blk.npz")))
IDS = [os.path.basename(p)[:-len("_blk.npz")] for p in BLK]


def load(p):
    z = np.load(p)
    return {k: z[k] for k in z.files}


def test_blocking_fixtures_exist():
    assert BLK, "no *_blk.npz fixtures"
    ds = [load(p) for p in BLK]
    assert any(int(d["right"]) == 0 for d in ds) or any(int(d["right"]) == 1 for d in ds)


@pytest.mark.parametrize("path", BLK, ids=IDS)
def test_oracle_replay_matches_reference_blocking(path):
    d = load(path)
    out = oracle.block_contract(d, d["env"], d["site"], int(d["tmp_size"]), d["out"].size)
    ref = d["out"]
    scale = max(1.0, float(np.abs(ref).max()))
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * scale)


@pytest.fixture(scope="module")
def ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from b2g.heff import Context
    c = Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", BLK, ids=IDS)
def test_gpu_blocking_matches_reference(ctx, path):
    from b2g.blocking import contract
    d = load(path)
    out = contract(ctx, d, d["env"], d["site"], int(d["tmp_size"]), d["out"].size)
    ref = d["out"]
    scale = max(1.0, float(np.abs(ref).max()))
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * scale)
    # reproducible bit for bit
    out2 = contract(ctx, d, d["env"], d["site"], int(d["tmp_size"]), d["out"].size)
    assert np.array_equal(out, out2)


@pytest.mark.gpu
@pytest.mark.parametrize("path", BLK, ids=IDS)
def test_gpu_blocking_device_resident(ctx, path):
    """b2g_block_contract_device (operands and output stay on the device) gives
    the host entry's result bit for bit; the output then serves as an
    operator blob on the device without a host round trip."""
    torch = pytest.importorskip("torch")
    from b2g.blocking import contract, contract_device
    d = load(path)
    host = contract(ctx, d, d["env"], d["site"], int(d["tmp_size"]), d["out"].size)
    env = torch.from_numpy(np.ascontiguousarray(d["env"], dtype=np.float64)).cuda()
    site = torch.from_numpy(np.ascontiguousarray(d["site"], dtype=np.float64)).cuda()
    out = torch.full((max(d["out"].size, 1),), 7.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    contract_device(ctx, d, env, site, int(d["tmp_size"]), out)
    ctx.synchronize()
    assert np.array_equal(out.cpu().numpy()[:d["out"].size], host)
