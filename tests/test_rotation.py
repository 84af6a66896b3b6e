"""Operator rotation (renormalisation) after a site: the reference's
TensorFunctions::left_rotate / right_rotate (src/core/tensor_functions.hpp:2365-2403)
recorded as GEMM pairs (work = A op(ket); C += op(bra) work, the order of
GMatrixFunctions::rotate, src/core/matrix_functions.hpp:998-1009) and replayed
by the same plan/kernels as H_eff*psi.  "psi" is the packed input operator
data, "ops" the MPS tensor, "sigma" the reference's rotated operators."""
import numpy as np
import pytest

from conftest import rotation_ids
from oracle import oracle


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", rotation_ids())
def test_oracle_rotation_matches_reference(problems, name):
    p = problems[name]
    out = oracle.replay(p.seq(), p.ops, p.psi, p.sigma_size, nthreads=2)
    assert rel(out, p.sigma) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", rotation_ids())
def test_gpu_rotation_matches_reference(problems, name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import b2g
    p = problems[name]
    ctx = b2g.Context(0)
    h = b2g.EffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
    x = torch.from_numpy(p.psi).cuda()
    for form, tol in ((b2g.FP64, 1e-12), (b2g.TF32X3, 2e-5)):
        y = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
        h(x, y, 1.0, form)
        h.status()
        assert rel(y.cpu().numpy(), p.sigma) <= tol, form
    h.close()
    ctx.close()
