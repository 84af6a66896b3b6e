"""Term-sharded H_eff*psi over ranks (one GPU per rank).

The reference distributes the terms of H_eff over MPI ranks (ParallelRuleQC,
src/dmrg/qc_parallel_rule.hpp:31-85); ParallelTensorFunctions::operator()
(src/core/parallel_tensor_functions.hpp:51-55) replays the rank's own
BatchGEMMSeq and sums sigma over the ranks with allreduce_sum.  Here every
rank keeps the recorded pairs that b2g_partition_pairs assigns it (pairs that
share a GEMM0 product stay together), builds its own device plan from them,
and the partial sigmas are summed with one all_reduce of the process group
(NCCL for device tensors, gloo for host arrays).

Difference kept on purpose: the reference all-reduces c after accumulating
into it, so a c that is not zero on entry is counted once per rank; here the
rank's share goes into a zeroed buffer that is reduced and then added, so
c += scale * H_eff * b holds for any c.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .capi import FP64, PairSeq, check, lib


def partition_pairs(seq: PairSeq, n_ranks: int):
    """(rank_of_pair int32[n_pairs], load float64[n_ranks]) from b2g_partition_pairs."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be >= 1")
    rank_of = np.zeros(seq.n, dtype=np.int32)
    load = np.zeros(n_ranks)
    check(lib().b2g_partition_pairs(C.byref(seq.c), n_ranks, rank_of.ctypes.data,
                                    load.ctypes.data))
    return rank_of, load


def rank_pairs(seq: PairSeq, n_ranks: int, rank: int) -> PairSeq:
    """The pairs of rank `rank` (in recorded order) as their own sequence."""
    if not 0 <= rank < n_ranks:
        raise ValueError("rank out of range")
    rank_of, _ = partition_pairs(seq, n_ranks)
    return seq.subset(np.nonzero(rank_of == rank)[0])


class ShardedEffectiveHamiltonian:
    """H_eff whose pairs are split over the ranks of a torch.distributed group.

    engine: the class that builds and applies one rank's share (default
    b2g.EffectiveHamiltonian; same constructor and call signature).
    """

    def __init__(self, ctx, seq, ops, psi_size: int, sigma_size: int, group=None, engine=None):
        import torch.distributed as dist

        if engine is None:
            from .heff import EffectiveHamiltonian as engine
        if not isinstance(seq, PairSeq):
            seq = PairSeq(seq)
        self.group = group
        self.rank = dist.get_rank(group)
        self.n_ranks = dist.get_world_size(group)
        rank_of, self.load = partition_pairs(seq, self.n_ranks)
        self.local_seq = seq.subset(np.nonzero(rank_of == self.rank)[0])
        self.psi_size, self.sigma_size = int(psi_size), int(sigma_size)
        self.local = engine(ctx, self.local_seq, ops, psi_size, sigma_size)

    def __call__(self, b, c, scale: float = 1.0, form: int = FP64):
        """c += scale * H_eff * b, summed over the ranks (every rank gets the sum)."""
        import torch
        import torch.distributed as dist

        if isinstance(c, np.ndarray):
            part = np.zeros_like(c)
            self.local(b, part, scale, form)
            t = torch.from_numpy(part)
            dist.all_reduce(t, group=self.group)
            c += part
        else:
            part = torch.zeros_like(c)
            if part.is_cuda:
                # the zero-fill (and whatever torch last wrote into b) runs on
                # torch's current stream; the library launches on its own
                # context stream, so finish torch's work first
                torch.cuda.current_stream(part.device).synchronize()
            self.local(b, part, scale, form)
            if part.is_cuda:
                # the rank's kernels run on the context stream: finish them
                # before the collective reads the buffer
                self.local.ctx.synchronize()
            dist.all_reduce(part, group=self.group)
            c.add_(part)
        return c

    def adjoint(self, x, y, grad_ops=None, grad_psi=None, scale: float = 1.0):
        """Gradients of <x|H_eff|y> summed over the ranks: each rank
        differentiates its own pairs into zeroed buffers, one all_reduce per
        gradient, then grad += the sum (every rank gets it).  Host numpy
        arrays (gloo) or CUDA tensors (NCCL), matching the engine."""
        import torch
        import torch.distributed as dist

        host = isinstance(x, np.ndarray)
        parts = []
        for g in (grad_ops, grad_psi):
            if g is None:
                parts.append(None)
            else:
                parts.append(np.zeros_like(g) if host else torch.zeros_like(g))
        if not host:
            # zero-fills and torch's writes to x, y run on torch's current
            # stream, the adjoint kernels on the library's context stream
            torch.cuda.current_stream(x.device).synchronize()
        self.local.adjoint(x, y, parts[0], parts[1], scale)
        if not host and hasattr(self.local, "ctx"):
            self.local.ctx.synchronize()
        for g, part in zip((grad_ops, grad_psi), parts):
            if g is None:
                continue
            t = torch.from_numpy(part) if host else part
            dist.all_reduce(t, group=self.group)
            if host:
                g += part
            else:
                g.add_(part)

    def close(self):
        if hasattr(self.local, "close"):
            self.local.close()
