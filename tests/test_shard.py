"""A pass split over several devices (root partition + sum of the per-shard
n-vectors).  Root edges are independent within a pass, so the sum of the
shards' increments must equal the unsplit pass exactly.

The CPU test runs two gloo ranks: each takes its share of roots from the
library's partition (host code), computes its shard with the oracle, and the
ranks all-reduce.  The GPU test runs the shards of the library itself one
after another on one device (the ranks would wait on nothing of each other).
"""
import os
import socket

import numpy as np
import pytest

import kclistpp_gb300 as K
from oracle import oracle as O

WORLD = 2


def _graph_pairs():
    return K.planted(3000, 6.0, 2.2, 2, 90, 160, 0.5, seed=31).pairs()


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_shard_plan_covers_every_root_once():
    og = O.Graph(_graph_pairs())
    off, _ = og.csr()
    deg = np.diff(off)
    for world in (1, 2, 3, 8):
        owner = K.shard_plan(off, world)
        assert owner.shape == (og.n,)
        assert owner.max() < world
        if world > 1:
            load = np.bincount(owner[deg > 0], weights=(deg[deg > 0].astype(float) ** 2), minlength=world)
            assert load.max() <= 1.25 * load.mean() + deg.max() ** 2  # greedy balance


def _rank_main(rank: int, port: int, result_path: str):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    P = _graph_pairs()
    og = O.Graph(P)
    off, _ = og.csr()
    owner = K.shard_plan(off, WORLD)
    mask = (owner == rank).astype(np.uint8)
    rng = np.random.default_rng(5)
    r = rng.integers(0, 3, size=og.n, dtype=np.uint64)
    rho = rng.integers(0, 3, size=og.n).astype(np.float64) * 0.5
    ok = True
    for k in (3, 4, 5):
        d = torch.from_numpy(og.seq_delta_masked(k, r, mask).astype(np.int64))
        dist.all_reduce(d)
        full = og.seq_pass(k, r, mode=O.SEQ_EDGE_STREAMS)
        ok &= np.array_equal(r + d.numpy().astype(np.uint64), full)
        c = torch.from_numpy(og.sim_counts_masked(k, rho, mask).astype(np.int64))
        dist.all_reduce(c)
        ok &= np.array_equal(c.numpy().astype(np.uint64), og.sim_counts(k, rho))
    if rank == 0:
        with open(result_path, "w") as f:
            f.write("ok" if ok else "mismatch")
    dist.barrier()
    dist.destroy_process_group()


def test_split_pass_sums_to_the_whole_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    out = str(tmp_path / "result")
    mp.spawn(_rank_main, args=(_free_port(), out), nprocs=WORLD, join=True)
    assert open(out).read() == "ok"


@pytest.mark.gpu
def test_split_pass_on_gpu(ctx):
    torch = pytest.importorskip("torch")
    P = _graph_pairs()
    g = K.build_graph(ctx, K.EdgeList.from_pairs(P))
    n = g.n
    rng = np.random.default_rng(6)
    r0 = rng.integers(0, 3, size=n, dtype=np.uint64)
    rho0 = rng.integers(0, 3, size=n).astype(np.float64) * 0.5
    for k in (3, 4, 5):
        full_r = K.seq_passes(g, k, 1, r0)
        full_c = K.sim_counts(g, k, rho0)
        r_d = torch.from_numpy(r0.view(np.int64).copy()).cuda()
        rho_d = torch.from_numpy(rho0.copy()).cuda()
        acc_r = torch.zeros(n, dtype=torch.int64, device="cuda")
        acc_c = torch.zeros(n, dtype=torch.int64, device="cuda")
        part = torch.empty(n, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()  # the library runs on its own stream
        for rank in range(WORLD):
            K.graph_shard(g, rank, WORLD)
            K.seq_delta_dev(g, k, r_d.data_ptr(), part.data_ptr())
            ctx.synchronize()
            acc_r += part
            torch.cuda.synchronize()
            K.sim_counts_dev(g, k, rho_d.data_ptr(), part.data_ptr())
            ctx.synchronize()
            acc_c += part
            torch.cuda.synchronize()
        # a whole-graph entry point refuses a sharded graph (its result would be partial)
        with pytest.raises(K.KclppError) as e:
            K.seq_passes(g, k, 1, r0)
        assert e.value.status == K.ERR_INVALID and b"sharded" in K._lib.kclpp_last_error()
        K.graph_shard(g, 0, 1)
        assert np.array_equal(r0 + acc_r.cpu().numpy().view(np.uint64), full_r)
        assert np.array_equal(acc_c.cpu().numpy().view(np.uint64), full_c)
        # the Sim update on the summed counts equals the unsplit pass
        torch.cuda.synchronize()
        K.sim_update_dev(ctx, n, 1, rho_d.data_ptr(), acc_c.data_ptr())
        ctx.synchronize()
        assert np.array_equal(rho_d.cpu().numpy().view(np.uint64), K.sim_passes(g, k, 1, rho0).view(np.uint64))
