"""Host-side mirror of block2's EffectiveHamiltonian for the GB300 path.

The reference builds one EffectiveHamiltonian per site
(src/dmrg/effective_hamiltonian.hpp:99-1160): ``precompute`` records the GEMM
pairs of H_eff*psi into BatchGEMMSeq, the Davidson operator replays them
through ``TensorFunctions::operator()(b, c, scale)`` (c += scale * H b), and
``eigs`` returns (energy, ndav, nflop, tdav).  This class keeps those names
and meanings; the recorded pairs and the operator blob become a device plan
(b2g_heff_create), every product runs on the GPU (b2g_heff_apply), and
Davidson runs device-resident (b2g_davidson).  Errors surface as B2GError
(the reference throws std::runtime_error).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import capi
from .capi import FP32, FP64, TF32X3, B2GError, PairSeq, check, lib


class Context:
    """One device context (b2g_context): the device and the stream kernels run on."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        check(lib().b2g_context_create(device, C.byref(self._h)))
        self.device = device

    @property
    def handle(self):
        return self._h

    @property
    def stream_ptr(self) -> int:
        return lib().b2g_context_stream(self._h) or 0

    def synchronize(self):
        check(lib().b2g_context_synchronize(self._h))

    def close(self):
        if self._h:
            lib().b2g_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ptr(x):
    """Raw data pointer of a numpy array or a torch tensor."""
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


class EffectiveHamiltonian:
    """Device plan of one H_eff built from its recorded pair sequence.

    seq: PairSeq (or dict of arrays) -- BatchGEMMSeq batch[0]/batch[1] pairs
    ops: float64 operator blob (numpy, host) the pair offsets index
    psi_size / sigma_size: lengths of the ket / bra wavefunctions
    """

    def __init__(self, ctx: Context, seq, ops, psi_size: int, sigma_size: int):
        if not isinstance(seq, PairSeq):
            seq = PairSeq(seq)
        self.ctx = ctx
        self.seq = seq
        ops = np.ascontiguousarray(ops, dtype=np.float64)
        self.psi_size, self.sigma_size = int(psi_size), int(sigma_size)
        self.ops_size = int(ops.size)
        self._adjoint_ready = False
        self._h = C.c_void_p()
        check(lib().b2g_heff_create(ctx.handle, C.byref(seq.c), ops.ctypes.data, ops.size, 0,
                                    self.psi_size, self.sigma_size, C.byref(self._h)))
        st = capi.HeffStatsC()
        check(lib().b2g_heff_stats_get(self._h, C.byref(st)))
        self.stats = st.as_dict()
        self.nflop = 2.0 * self.stats["mnk"]    # FLOP of one product (2 x reference mnk)

    # c += scale * H_eff * b   (TensorFunctions::operator(), tensor_functions.hpp:59-62)
    def __call__(self, b, c, scale: float = 1.0, form: int = FP64):
        if isinstance(b, np.ndarray) != isinstance(c, np.ndarray):
            raise TypeError("b and c must both be host numpy arrays or both device tensors")
        if isinstance(b, np.ndarray):
            if b.dtype != np.float64 or c.dtype != np.float64 or not c.flags.c_contiguous:
                raise TypeError("host buffers must be contiguous float64")
            if b.size != self.psi_size or c.size != self.sigma_size:
                raise ValueError("wavefunction sizes do not match the effective Hamiltonian")
            bb = np.ascontiguousarray(b)
            check(lib().b2g_heff_apply_host(self._h, bb.ctypes.data, c.ctypes.data, scale, form))
        else:
            if b.numel() != self.psi_size or c.numel() != self.sigma_size:
                raise ValueError("wavefunction sizes do not match the effective Hamiltonian")
            if not (b.is_cuda and c.is_cuda and b.is_contiguous() and c.is_contiguous()):
                raise TypeError("device buffers must be contiguous CUDA tensors")
            check(lib().b2g_heff_apply(self._h, _ptr(b), _ptr(c), scale, form))
        return c

    def apply_batch(self, b, c, scale: float = 1.0, form: int = FP64):
        """c[r] += scale * H_eff * b[r] for every row r of the (nroots, size)
        CUDA tensors b and c, in one launch per kernel."""
        if b.dim() != 2 or c.dim() != 2 or b.shape[0] != c.shape[0]:
            raise ValueError("b and c must be (nroots, size) tensors with equal nroots")
        if b.shape[1] != self.psi_size or c.shape[1] != self.sigma_size:
            raise ValueError("wavefunction sizes do not match the effective Hamiltonian")
        if not (b.is_cuda and c.is_cuda and b.is_contiguous() and c.is_contiguous()):
            raise TypeError("device buffers must be contiguous CUDA tensors")
        check(lib().b2g_heff_apply_batch(self._h, _ptr(b), _ptr(c), int(b.shape[0]), scale, form))
        return c

    # diag(H_eff): the reference builds it in the EffectiveHamiltonian ctor
    # (effective_hamiltonian.hpp:190-200); here it follows from the recorded pairs
    def diag(self, out=None):
        """diag(H_eff) as a float64 numpy array (out=None) or into the CUDA tensor out."""
        if out is None:
            d = np.zeros(self.sigma_size)
            check(lib().b2g_heff_diag_host(self._h, d.ctypes.data))
            return d
        if not (out.is_cuda and out.is_contiguous()) or out.numel() != self.sigma_size:
            raise ValueError("out must be a contiguous CUDA tensor of sigma_size doubles")
        check(lib().b2g_heff_diag(self._h, _ptr(out)))
        return out

    def autotune(self, form: int = TF32X3) -> dict:
        """Time the candidate tile shapes of this H_eff (from its block-size
        histogram) and keep the fastest plan; returns the candidates, their
        median apply times (ms) and the index kept."""
        res = capi.TuneResultC()
        check(lib().b2g_heff_autotune(self._h, C.byref(self.seq.c), form, C.byref(res)))
        return res.as_dict()

    @property
    def params(self) -> dict:
        """Tile shapes of the installed plan."""
        v = (C.c_int32 * 3)()
        check(lib().b2g_heff_get_params(self._h, v))
        return {"g0_tile_cols": v[0], "g1_tile_cols": v[1], "g1_chunk": v[2]}

    def set_params(self, g0_tile_cols: int, g1_tile_cols: int, g1_chunk: int):
        """Install the plan with these tile shapes (no timing)."""
        v = (C.c_int32 * 3)(g0_tile_cols, g1_tile_cols, g1_chunk)
        check(lib().b2g_heff_set_params(self._h, C.byref(self.seq.c), v))

    def set_graphs(self, enable: bool):
        """Replay repeated applies as CUDA graphs (default on); False drops them."""
        check(lib().b2g_heff_set_graphs(self._h, int(bool(enable))))

    @property
    def graph_count(self) -> int:
        """Captured apply graphs currently held."""
        return lib().b2g_heff_graph_count(self._h)

    def status(self):
        """Synchronize and raise if a tensor-core kernel gave up a bounded wait."""
        check(lib().b2g_heff_status(self._h))

    def apply_ptr(self, psi_ptr: int, sigma_ptr: int, scale: float = 1.0, form: int = FP64):
        """Raw device-pointer entry (asynchronous on the context stream)."""
        check(lib().b2g_heff_apply(self._h, psi_ptr, sigma_ptr, scale, form))

    # EffectiveHamiltonian::eigs (effective_hamiltonian.hpp:481-568) for one root
    def eigs(self, diag, psi, conv_thrd: float = 5e-6, max_iter: int = 5000,
             def_min: int = 2, def_max: int = 50, form: int = FP64):
        """Lowest eigenpair; psi (host float64) is the initial guess and is
        overwritten with the eigenvector.  Returns (energy, ndav, nflop, tdav)."""
        diag = np.ascontiguousarray(diag, dtype=np.float64)
        if psi.dtype != np.float64 or not psi.flags.c_contiguous:
            raise TypeError("psi must be a contiguous float64 array")
        res = capi.DavidsonResultC()
        t0 = time.perf_counter()
        rc = lib().b2g_davidson(self._h, diag.ctypes.data, psi.ctypes.data, conv_thrd, max_iter,
                                def_min, def_max, form, C.byref(res))
        tdav = time.perf_counter() - t0
        self.last_davidson = res   # also when the solve stops unconverged (max_iter)
        self.last_tdav = tdav
        check(rc)
        nflop = self.nflop * (res.n_apply_fp64 + res.n_apply_mixed)
        return res.energy, res.n_iter, nflop, tdav

    # EffectiveHamiltonian<S, FL, MultiMPS>::eigs (effective_hamiltonian.hpp:1711-1797)
    def eigs_multi(self, diag, psis, conv_thrd: float = 5e-6, max_iter: int = 5000,
                   def_min: int = 2, def_max: int = 50, form: int = FP64):
        """k lowest eigenpairs; psis (k, n) host float64 guesses, overwritten with
        the eigenvectors.  Returns (energies[k], ndav, nflop, tdav)."""
        diag = np.ascontiguousarray(diag, dtype=np.float64)
        if psis.dtype != np.float64 or not psis.flags.c_contiguous or psis.ndim != 2:
            raise TypeError("psis must be a contiguous (k, n) float64 array")
        k = psis.shape[0]
        energies = np.zeros(k)
        res = capi.DavidsonResultC()
        t0 = time.perf_counter()
        rc = lib().b2g_davidson_multi(self._h, diag.ctypes.data, psis.ctypes.data, k, conv_thrd,
                                      max_iter, def_min, def_max, form, energies.ctypes.data,
                                      C.byref(res))
        tdav = time.perf_counter() - t0
        check(rc)
        self.last_davidson = res
        return energies, res.n_iter, self.nflop * (res.n_apply_fp64 + res.n_apply_mixed), tdav

    # ---- differentiation form (no reference counterpart; see b2g.autodiff) ----
    def set_ops(self, ops):
        """Replace the operator values (same layout and size): a float64 numpy
        array (host, synchronous) or a contiguous float64 CUDA tensor (copied on
        the context stream)."""
        if isinstance(ops, np.ndarray):
            ops = np.ascontiguousarray(ops, dtype=np.float64)
            if ops.size != self.ops_size:
                raise ValueError("operator blob size does not match the effective Hamiltonian")
            check(lib().b2g_heff_set_ops(self._h, ops.ctypes.data, 0))
        else:
            if ops.numel() != self.ops_size:
                raise ValueError("operator blob size does not match the effective Hamiltonian")
            if not (ops.is_cuda and ops.is_contiguous()):
                raise TypeError("ops must be a contiguous CUDA tensor")
            check(lib().b2g_heff_set_ops(self._h, _ptr(ops), 1))

    def adjoint(self, x, y, grad_ops=None, grad_psi=None, scale: float = 1.0):
        """Gradients of f = <x| H_eff |y> (CUDA tensors, FP64):
        grad_ops += scale * df/dops, grad_psi += scale * H_eff^T x.  Either
        output may be None.  Asynchronous on the context stream."""
        if not self._adjoint_ready:
            check(lib().b2g_heff_adjoint_prepare(self._h, C.byref(self.seq.c)))
            self._adjoint_ready = True
        if x.numel() != self.sigma_size or (y is not None and y.numel() != self.psi_size):
            raise ValueError("bra/ket sizes do not match the effective Hamiltonian")
        if grad_ops is not None and grad_ops.numel() != self.ops_size:
            raise ValueError("grad_ops must hold ops_size doubles")
        if grad_psi is not None and grad_psi.numel() != self.psi_size:
            raise ValueError("grad_psi must hold psi_size doubles")
        for t in (x, y, grad_ops, grad_psi):
            if t is not None and not (t.is_cuda and t.is_contiguous()):
                raise TypeError("adjoint buffers must be contiguous CUDA tensors")
        check(lib().b2g_heff_adjoint(self._h, _ptr(x), None if y is None else _ptr(y), scale,
                                     None if grad_ops is None else _ptr(grad_ops),
                                     None if grad_psi is None else _ptr(grad_psi)))

    @property
    def adjoint_nflop(self) -> float:
        """FLOP of one adjoint with both gradients (2 x multiply-adds)."""
        if not self._adjoint_ready:
            check(lib().b2g_heff_adjoint_prepare(self._h, C.byref(self.seq.c)))
            self._adjoint_ready = True
        v = C.c_double()
        check(lib().b2g_heff_adjoint_mnk(self._h, C.byref(v)))
        return 2.0 * v.value

    def close(self):
        if self._h:
            lib().b2g_heff_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
