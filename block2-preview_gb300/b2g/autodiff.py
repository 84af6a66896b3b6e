"""Differentiation form: H_eff*psi and the converged site energy as
torch.autograd functions of the operator blob.

The reference has no adjoint of its contraction; it obtains energy
derivatives with respect to the Hamiltonian only as reduced density matrices
from expectation sweeps (src/dmrg/sweep_algorithm.hpp, class Expect).  Here
the effective Hamiltonian of one site is a function of its operator blob,
H_eff(ops) = sum_p alpha_p op(L_p) (.) op(R_p) over the recorded pairs
(BatchGEMMSeq::rotate semantics, src/core/batch_gemm.hpp:893-902; L_p and R_p
are both blocks of the blob, so H_eff is quadratic in it), and the
hand-written adjoint kernel (b2g_heff_adjoint) returns

  d<x|H_eff|y>/d ops   and   d<x|H_eff|y>/d y = H_eff^T x

in FP64.  For a converged eigenvector psi (normalised) of the symmetric
H_eff, the derivative of the lowest eigenvalue is psi^T (dH_eff/d ops) psi
(Hellmann-Feynman), i.e. the adjoint with x = y = psi.

All tensors are float64 CUDA tensors.  The library works on its own stream;
these functions synchronise torch's current stream before handing buffers
over and the library's stream before returning them.
"""
from __future__ import annotations

import numpy as np

try:
    import torch
except ImportError as e:  # pragma: no cover - torch is a hard dependency of this module
    raise ImportError("b2g.autodiff needs torch") from e

from .heff import EffectiveHamiltonian


def _to_lib(heff: EffectiveHamiltonian):
    torch.cuda.current_stream().synchronize()


def _from_lib(heff: EffectiveHamiltonian):
    heff.ctx.synchronize()


class HeffApply(torch.autograd.Function):
    """sigma = H_eff(ops) psi, differentiable in ops and psi."""

    @staticmethod
    def forward(ctx, ops, psi, heff):
        psi = psi.contiguous()
        sigma = torch.zeros(heff.sigma_size, dtype=torch.float64, device=psi.device)
        _to_lib(heff)
        heff.set_ops(ops)
        heff(psi, sigma)
        _from_lib(heff)
        ctx.heff = heff
        ctx.save_for_backward(ops, psi)
        return sigma

    @staticmethod
    def backward(ctx, gsigma):
        ops, psi = ctx.saved_tensors
        heff = ctx.heff
        want_ops, want_psi = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        gops = torch.zeros_like(ops) if want_ops else None
        gpsi = torch.zeros_like(psi) if want_psi else None
        if want_ops or want_psi:
            g = gsigma.contiguous()
            _to_lib(heff)
            heff.set_ops(ops)  # another forward may have installed other values
            heff.adjoint(g, psi, gops, gpsi)
            _from_lib(heff)
        return gops, gpsi, None


def heff_apply(heff: EffectiveHamiltonian, ops, psi):
    """H_eff(ops) psi with gradients for ops and psi."""
    return HeffApply.apply(ops, psi, heff)


def rayleigh_energy(heff: EffectiveHamiltonian, ops, psi):
    """<psi|H_eff(ops)|psi> / <psi|psi>, differentiable in ops and psi."""
    return torch.dot(psi, heff_apply(heff, ops, psi)) / torch.dot(psi, psi)


class ConvergedEnergy(torch.autograd.Function):
    """Lowest eigenvalue of H_eff(ops) by the device Davidson (FP64), with the
    Hellmann-Feynman gradient psi^T (dH_eff/d ops) psi from the adjoint kernel.
    Returns (energy, eigenvector); the eigenvector carries no gradient."""

    @staticmethod
    def forward(ctx, ops, heff, psi0, conv_thrd, max_iter):
        _to_lib(heff)
        heff.set_ops(ops)
        diag = heff.diag()
        psi = np.array(psi0, dtype=np.float64, copy=True)
        e, _, _, _ = heff.eigs(diag, psi, conv_thrd=conv_thrd, max_iter=max_iter)
        v = torch.from_numpy(psi / np.linalg.norm(psi)).to(ops.device)
        ctx.heff = heff
        ctx.save_for_backward(ops, v)
        ctx.mark_non_differentiable(v)
        return ops.new_tensor(e), v

    @staticmethod
    def backward(ctx, ge, gv):
        ops, v = ctx.saved_tensors
        heff = ctx.heff
        gops = None
        if ctx.needs_input_grad[0]:
            gops = torch.zeros_like(ops)
            _to_lib(heff)
            heff.set_ops(ops)
            heff.adjoint(v, v, gops, None, scale=float(ge))
            _from_lib(heff)
        return gops, None, None, None, None


def converged_energy(heff: EffectiveHamiltonian, ops, psi0, conv_thrd: float = 1e-12,
                     max_iter: int = 5000):
    """(E, psi) of the lowest eigenpair of H_eff(ops); E is differentiable in ops.
    psi0: host float64 initial guess (not modified)."""
    return ConvergedEnergy.apply(ops, heff, psi0, conv_thrd, max_iter)


def chain_to_parameters(grad_ops, jac_idx, jac_val, jac_ptr):
    """dE/dtheta_k = sum_i dE/dops_i dops_i/dtheta_k for Jacobian columns stored
    sparse (column k: entries [jac_ptr[k], jac_ptr[k + 1]) of jac_idx / jac_val),
    e.g. the integral -> operator Jacobian of the MPO and environment
    construction at fixed MPS.  Returns a float64 numpy array (summed on the
    host in column order: deterministic)."""
    g = grad_ops.detach().cpu().numpy() if hasattr(grad_ops, "detach") else np.asarray(grad_ops)
    jac_idx, jac_val, jac_ptr = np.asarray(jac_idx), np.asarray(jac_val), np.asarray(jac_ptr)
    return np.array([float(g[jac_idx[a:b]] @ jac_val[a:b]) for a, b in zip(jac_ptr[:-1], jac_ptr[1:])])
