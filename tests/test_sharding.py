"""Term-sharded H_eff*psi: the partition (b2g_partition_pairs, host only), the
sum of the ranks' shares against the reference's sigma, and the collective
path over world_size-2 gloo ranks on the CPU (each rank replays its share
with the oracle), as the reference's ParallelTensorFunctions::operator()
(src/core/parallel_tensor_functions.hpp:51-55) sums sigma with allreduce_sum."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, fixture_ids

import b2g  # noqa: E402
from b2g.sharding import ShardedEffectiveHamiltonian, partition_pairs, rank_pairs  # noqa: E402
from oracle import oracle  # noqa: E402

RTOL = 1e-12


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def product_keys(seq):
    a = seq.arrays
    return list(zip(a["a0"].tolist(), a["b0"].tolist(), a["m0"].tolist(), a["n0"].tolist(),
                    a["k0"].tolist(), a["lda0"].tolist(), a["ldb0"].tolist(),
                    (a["tb0"] != 0).tolist()))


@pytest.mark.parametrize("name", fixture_ids())
@pytest.mark.parametrize("n_ranks", [1, 2, 3, 8])
def test_partition_keeps_products_together_and_balances(problems, name, n_ranks):
    seq = problems[name].seq()
    rank_of, load = partition_pairs(seq, n_ranks)
    assert rank_of.shape == (seq.n,) and rank_of.min() >= 0 and rank_of.max() < n_ranks
    owner, cost = {}, {}
    a = seq.arrays
    for i, k in enumerate(product_keys(seq)):
        assert owner.setdefault(k, rank_of[i]) == rank_of[i]
        if k not in cost:
            cost[k] = float(a["m0"][i]) * a["n0"][i] * a["k0"][i]
        cost[k] += float(a["m1"][i]) * a["n1"][i] * a["k1"][i]
    want = np.zeros(n_ranks)
    for k, r in owner.items():
        want[r] += cost[k]
    np.testing.assert_allclose(load, want, rtol=1e-12)
    # largest-first greedy: no rank exceeds the mean by more than the largest product
    assert load.max() <= load.sum() / n_ranks + max(cost.values()) + 1e-6
    again, _ = partition_pairs(seq, n_ranks)
    assert np.array_equal(again, rank_of)


def test_partition_rejects_bad_arguments(problems):
    import ctypes as C
    seq = problems[fixture_ids()[0]].seq()
    out = np.zeros(seq.n, dtype=np.int32)
    assert b2g.lib().b2g_partition_pairs(None, 2, out.ctypes.data, None) == 1
    assert b2g.lib().b2g_partition_pairs(C.byref(seq.c), 0, out.ctypes.data, None) == 1
    assert b2g.lib().b2g_partition_pairs(C.byref(seq.c), 2, None, None) == 1
    with pytest.raises(ValueError):
        partition_pairs(seq, 0)
    with pytest.raises(ValueError):
        rank_pairs(seq, 2, 2)


@pytest.mark.parametrize("name", fixture_ids())
@pytest.mark.parametrize("n_ranks", [2, 3])
def test_sum_of_rank_shares_matches_reference(problems, name, n_ranks):
    p = problems[name]
    seq = p.seq()
    total = np.zeros(p.sigma_size)
    n = 0
    for r in range(n_ranks):
        sub = rank_pairs(seq, n_ranks, r)
        n += sub.n
        total += oracle.replay(sub, p.ops, p.psi, p.sigma_size)
    assert n == seq.n
    assert rel(total, p.sigma) <= RTOL


class OracleShare:
    """One rank's share replayed on the CPU by the oracle (test stand-in for the GPU engine)."""

    def __init__(self, ctx, seq, ops, psi_size, sigma_size):
        self.seq, self.ops, self.sigma_size = seq, ops, sigma_size

    def __call__(self, b, c, scale=1.0, form=b2g.FP64):
        oracle.replay(self.seq, self.ops, b, self.sigma_size, scale, sigma=c)
        return c

    def adjoint(self, x, y, grad_ops, grad_psi, scale=1.0):
        go, gy = oracle.adjoint(self.seq, self.ops, x, y)
        if grad_ops is not None:
            grad_ops += scale * go
        if grad_psi is not None:
            grad_psi += scale * gy


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _gloo_rank(rank, world, port, name, out_dir):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from b2g.problem import load_problem
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p = load_problem(os.path.join(ROOT, "tests", "golden", name + ".npz"))
        h = ShardedEffectiveHamiltonian(None, p.seq(), p.ops, p.psi_size, p.sigma_size,
                                        engine=OracleShare)
        c = np.full(p.sigma_size, 0.25)   # c += scale * H psi keeps what c held
        h(p.psi, c, scale=0.5)
        np.save(os.path.join(out_dir, f"sigma{rank}.npy"), c)
        # the adjoint of the sharded product: one all_reduce per gradient
        x = np.random.default_rng(2).standard_normal(p.sigma_size)
        go, gy = np.zeros(p.ops.size), np.ones(p.psi_size)
        h.adjoint(x, p.psi, go, gy, scale=2.0)
        np.save(os.path.join(out_dir, f"gops{rank}.npy"), go)
        np.save(os.path.join(out_dir, f"gpsi{rank}.npy"), gy)
        np.save(os.path.join(out_dir, f"npairs{rank}.npy"), np.array([h.local_seq.n]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("name", ["hub8_su2", "syn8_sz"])
def test_gloo_two_ranks_sum_sigma(problems, name, tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    p = problems[name]
    port = _free_port()
    mp.start_processes(_gloo_rank, args=(2, port, name, str(tmp_path)), nprocs=2,
                       start_method="spawn", join=True)
    want = 0.25 + 0.5 * p.sigma
    got = [np.load(tmp_path / f"sigma{r}.npy") for r in range(2)]
    npairs = sum(int(np.load(tmp_path / f"npairs{r}.npy")[0]) for r in range(2))
    assert npairs == p.seq().n
    assert np.array_equal(got[0], got[1])
    assert rel(got[0], want) <= RTOL
    x = np.random.default_rng(2).standard_normal(p.sigma_size)
    go, gy = oracle.adjoint(p.seq(), p.ops, x, p.psi)
    for r in range(2):
        assert rel(np.load(tmp_path / f"gops{r}.npy"), 2.0 * go) <= RTOL
        assert rel(np.load(tmp_path / f"gpsi{r}.npy"), 1.0 + 2.0 * gy) <= RTOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", fixture_ids())
def test_gpu_rank_shares_sum_to_reference(problems, name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    p = problems[name]
    seq = p.seq()
    ctx = b2g.Context(0)
    try:
        psi = torch.from_numpy(p.psi).cuda()
        total = torch.zeros(p.sigma_size, dtype=torch.float64, device="cuda")
        for r in range(2):
            h = b2g.EffectiveHamiltonian(ctx, rank_pairs(seq, 2, r), p.ops, p.psi_size,
                                         p.sigma_size)
            h(psi, total)
            h.status()
            h.close()
        assert rel(total.cpu().numpy(), p.sigma) <= RTOL
    finally:
        ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hub8_su2", "syn8_sz"])
def test_gpu_rank_adjoint_shares_sum_to_full_adjoint(problems, name):
    """The adjoint of each rank's pairs (two shares built and run one after the
    other on one GPU) sums to the adjoint of the whole H_eff."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    p = problems[name]
    seq = p.seq()
    ctx = b2g.Context(0)
    x = np.random.default_rng(3).standard_normal(p.sigma_size)
    xd, yd = torch.from_numpy(x).cuda(), torch.from_numpy(p.psi).cuda()
    go = torch.zeros(p.ops.size, dtype=torch.float64, device="cuda")
    gy = torch.zeros(p.psi_size, dtype=torch.float64, device="cuda")
    for r in range(2):
        h = b2g.EffectiveHamiltonian(ctx, rank_pairs(seq, 2, r), p.ops, p.psi_size, p.sigma_size)
        torch.cuda.synchronize()
        h.adjoint(xd, yd, go, gy)
        ctx.synchronize()
        h.close()
    ref_o, ref_y = oracle.adjoint(seq, p.ops, x, p.psi)
    assert rel(go.cpu().numpy(), ref_o) <= RTOL
    assert rel(gy.cpu().numpy(), ref_y) <= RTOL
    ctx.close()


def _cuda_single_rank(rank, port, name, out_dir):
    """One rank of a single-rank NCCL group driving ShardedEffectiveHamiltonian
    on CUDA tensors with no synchronisation of its own: torch writes the
    inputs on its current stream and the class must order the library's
    context stream after them."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "block2-preview_gb300"))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    from b2g.problem import load_problem
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), NCCL_NVLS_ENABLE="0")
    torch.cuda.set_device(0)
    dist.init_process_group("nccl", rank=0, world_size=1)
    try:
        p = load_problem(os.path.join(ROOT, "tests", "golden", name + ".npz"))
        ctx = b2g.Context(0)
        h = ShardedEffectiveHamiltonian(ctx, p.seq(), p.ops, p.psi_size, p.sigma_size)
        psi = torch.from_numpy(p.psi).cuda() * 1.0          # written by a torch kernel
        c = torch.full((p.sigma_size,), 0.25, dtype=torch.float64, device="cuda")
        h(psi, c, scale=0.5)
        x = torch.from_numpy(np.random.default_rng(2).standard_normal(p.sigma_size)).cuda() * 1.0
        go = torch.zeros(p.ops.size, dtype=torch.float64, device="cuda")
        gy = torch.ones(p.psi_size, dtype=torch.float64, device="cuda")
        h.adjoint(x, psi, go, gy, scale=2.0)
        np.save(os.path.join(out_dir, "sigma.npy"), c.cpu().numpy())
        np.save(os.path.join(out_dir, "gops.npy"), go.cpu().numpy())
        np.save(os.path.join(out_dir, "gpsi.npy"), gy.cpu().numpy())
        h.close()
        ctx.close()
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hub8_su2", "syn8_sz"])
def test_gpu_sharded_class_orders_streams(problems, name, tmp_path):
    """ShardedEffectiveHamiltonian.__call__ and .adjoint on CUDA tensors, with
    no manual synchronisation in the caller, equal the reference's sigma and
    the oracle's adjoint."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mp = pytest.importorskip("torch.multiprocessing")
    p = problems[name]
    mp.start_processes(_cuda_single_rank, args=(_free_port(), name, str(tmp_path)), nprocs=1,
                       start_method="spawn", join=True)
    assert rel(np.load(tmp_path / "sigma.npy"), 0.25 + 0.5 * p.sigma) <= RTOL
    x = np.random.default_rng(2).standard_normal(p.sigma_size)
    go, gy = oracle.adjoint(p.seq(), p.ops, x, p.psi)
    assert rel(np.load(tmp_path / "gops.npy"), 2.0 * go) <= RTOL
    assert rel(np.load(tmp_path / "gpsi.npy"), 1.0 + 2.0 * gy) <= RTOL
