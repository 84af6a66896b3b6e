"""PDM fast expectations on the GPU (b2g.npdm.PdmSite): the partials' pairs
run by the H_eff engine must give the reference's partials and expectation
values (FP64 to 1e-12, TF32x3 to 2e-5 relative on the partials).

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
