"""diag(H_eff) on the GPU from the recorded pairs, against the diagonal the
reference builds in its EffectiveHamiltonian constructor (stored in every
golden fixture) and against the oracle's replay of unit vectors."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import fixture_ids


@pytest.fixture(scope="module")
def ctx():
    from b2g.heff import Context
    c = Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", fixture_ids())
def test_diag_matches_reference(ctx, problems, name):
    from b2g.heff import EffectiveHamiltonian
    prob = problems[name]
    h = EffectiveHamiltonian(ctx, prob.seq(), prob.ops, prob.psi_size, prob.sigma_size)
    d = h.diag()
    ref = np.asarray(prob.diag)
    np.testing.assert_allclose(d, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    # device-pointer entry gives the same bits
    import torch
    out = torch.zeros(prob.sigma_size, dtype=torch.float64, device="cuda")
    h.diag(out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), d)
    h.close()


def test_diag_identity_on_oracle(problems):
    """The identity the GPU kernel uses, checked on the CPU: the reference's
    diagonal equals e_x . H e_x for sampled x, with H applied by the oracle's
    replay of the recorded pairs."""
    from oracle import oracle
    prob = problems["hub8_su2"]
    rng = np.random.default_rng(5)
    for x in rng.choice(prob.psi_size, size=8, replace=False):
        e = np.zeros(prob.psi_size)
        e[x] = 1.0
        s = oracle.replay(prob.seq(), prob.ops, e, prob.sigma_size)
        assert s[x] == pytest.approx(prob.diag[x], rel=1e-12, abs=1e-14)
