"""PDM fast expectations on the GPU (b2g.npdm.PdmSite): the partials' pairs
run by the H_eff engine must give the reference's partials and expectation
values (FP64 to 1e-12, TF32x3 to 2e-5 relative on the partials).

Through block2's own Expect sweep (the sweep program's --pdm 2): the GPU arm's
1-PDM, whose fast-expectation partials run on the device
(GpuTensorFunctions::tensor_product_expectation), equals block2's 1-PDM of the
same MPS to 1e-12.

This file is collected after the other GPU tests."""
import numpy as np
import pytest

from conftest import npdm_ids
import b2g
from b2g.npdm import PdmSite
from npdm_fixture import load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", npdm_ids())
def test_gpu_pdm_site_matches_reference(name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    d = load(name)
    ctx = b2g.Context(0)
    site = PdmSite(ctx, d["seq"], d["psi"], d["ops"], d["sigma"].size, d["layout"], d["terms"], d["rmats"],
                   d["meta"]["n_expect"])
    scale = max(np.linalg.norm(d["sigma"]), 1e-300)
    emax = max(np.abs(d["expect"]).max(), 1.0)
    for form, tol in ((b2g.FP64, 1e-12), (b2g.TF32X3, 2e-5)):
        p = site.partials(form)
        assert np.linalg.norm(p - d["sigma"]) / scale <= tol, form
        assert np.abs(site.values(form) - d["expect"]).max() <= tol * emax, form
    site.close()
    ctx.close()


@pytest.mark.gpu
def test_gpu_pdm_in_block2_expect_sweep(tmp_path):
    import os
    from b2g.sweep import SWEEP_BIN, run_sweep
    from test_npdm import HUB8_PDM
    if not os.path.exists(SWEEP_BIN):
        pytest.skip("sweep program not built (no block2 headers)")
    r = run_sweep(binary=SWEEP_BIN, arms=("gpu:fp64",), threads=4, workdir=str(tmp_path),
                  **dict(HUB8_PDM, pdm=2))
    arm = r["arms"][0]
    assert arm["pdm1_device_products"] > 0
    dev, host = np.array(arm["pdm1"]), np.array(arm["pdm1_host"])
    assert np.abs(dev - host).max() <= 1e-12, np.abs(dev - host).max()
    assert abs(np.trace(dev.reshape(8, 8)) - 8.0) < 1e-10
