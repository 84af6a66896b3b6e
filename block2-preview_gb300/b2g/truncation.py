"""Host-side mirror of block2's density-matrix truncation for the GB300 path.

After Davidson, the reference's two-site blocking (src/dmrg/sweep_algorithm.hpp:
410-445) forms the reduced density matrix of the converged wavefunction
(MovingEnvironment::density_matrix, src/dmrg/moving_environment.hpp:3554-3580),
keeps its largest eigenvalues (truncate_density_matrix, 3715-3843) and splits
the wavefunction into the new MPS tensor and the carried wavefunction
(split_density_matrix, 4250-4345).  ``split_density_matrix`` below keeps that
name and argument meaning (k = bond dimension, -1 keeps all; trace_right =
forward sweep; cutoff) and runs the density matrix and its eigen-
decomposition on the GPU (b2g_dm_truncate).  Errors surface as B2GError.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from .capi import DmLayoutC, DmResultC, check, lib


@dataclass
class DensityMatrixLayout:
    """Block layout of a two-site wavefunction and its density matrix.

    psi_rows/psi_cols/psi_off: the wavefunction's blocks (row-major);
    psi_dm: the density-matrix block each one contributes to (-1: none);
    dm_dim: the sizes of the density-matrix blocks; trace_right: trace out
    the right index (forward sweep)."""
    trace_right: bool
    psi_dm: np.ndarray
    psi_rows: np.ndarray
    psi_cols: np.ndarray
    psi_off: np.ndarray
    dm_dim: np.ndarray

    def __post_init__(self):
        self.psi_dm = np.ascontiguousarray(self.psi_dm, dtype=np.int32)
        self.psi_rows = np.ascontiguousarray(self.psi_rows, dtype=np.int32)
        self.psi_cols = np.ascontiguousarray(self.psi_cols, dtype=np.int32)
        self.psi_off = np.ascontiguousarray(self.psi_off, dtype=np.uint64)
        self.dm_dim = np.ascontiguousarray(self.dm_dim, dtype=np.int32)

    @property
    def psi_size(self) -> int:
        if self.psi_rows.size == 0:
            return 0
        return int((self.psi_off + self.psi_rows.astype(np.uint64) * self.psi_cols).max())

    def c(self) -> DmLayoutC:
        return DmLayoutC(int(bool(self.trace_right)), self.psi_dm.size, self.psi_dm.ctypes.data,
                         self.psi_rows.ctypes.data, self.psi_cols.ctypes.data,
                         self.psi_off.ctypes.data, self.dm_dim.size, self.dm_dim.ctypes.data)


@dataclass
class SplitResult:
    eigenvalues: list      # per dm block, ascending
    kept: np.ndarray       # states kept per dm block
    rotation: list         # per dm block with kept states: the MPS tensor block
    wavefunction: list     # per psi block (None where its dm block keeps nothing)
    error: float           # discarded weight

    @property
    def n_kept(self) -> int:
        return int(self.kept.sum())


def split_density_matrix(ctx, layout: DensityMatrixLayout, psi, k: int, cutoff: float = 0.0
                         ) -> SplitResult:
    """MovingEnvironment::split_density_matrix (Physical truncation,
    normalize = True) with rho and its eigenvectors computed on the GPU.

    trace_right: rotation blocks are dm_dim x kept (the left MPS tensor) and
    the wavefunction blocks rot^T psi_a; otherwise rotation blocks are
    kept x dm_dim (the right MPS tensor) and the wavefunction psi_a rot^T."""
    psi = np.ascontiguousarray(psi, dtype=np.float64)
    if psi.size < layout.psi_size:
        raise ValueError("psi is shorter than its block layout")
    dims = layout.dm_dim.astype(np.int64)
    eig = np.zeros(max(int(dims.sum()), 1))
    kept = np.zeros(max(dims.size, 1), dtype=np.int32)
    rot = np.zeros(max(int((dims * dims).sum()), 1))
    wfn = np.zeros(max(psi.size, 1))
    res = DmResultC()
    lay = layout.c()
    check(lib().b2g_dm_truncate(ctx.handle, C.byref(lay), psi.ctypes.data, int(k), float(cutoff),
                                eig.ctypes.data, kept.ctypes.data, rot.ctypes.data,
                                wfn.ctypes.data, C.byref(res)))
    kept = kept[:dims.size].copy()
    eigs, rots, pos, rpos = [], [], 0, 0
    for b, n in enumerate(dims):
        eigs.append(eig[pos:pos + n].copy())
        pos += n
        im = int(kept[b])
        shape = (int(n), im) if layout.trace_right else (im, int(n))
        rots.append(rot[rpos:rpos + n * im].reshape(shape).copy() if im else None)
        rpos += n * im
    wfns, wpos = [], 0
    for a in range(layout.psi_dm.size):
        b = int(layout.psi_dm[a])
        if b < 0 or kept[b] == 0:
            wfns.append(None)
            continue
        im = int(kept[b])
        r, c = int(layout.psi_rows[a]), int(layout.psi_cols[a])
        shape = (im, c) if layout.trace_right else (r, im)
        wfns.append(wfn[wpos:wpos + shape[0] * shape[1]].reshape(shape).copy())
        wpos += shape[0] * shape[1]
    return SplitResult(eigs, kept, rots, wfns, float(res.error))
