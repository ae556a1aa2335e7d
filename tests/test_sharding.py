"""Multi-GPU path of the independent-model workloads, on CPU: models split
across ranks by cost, solved per rank, results gathered on rank 0 over gloo
(world size 2).  The per-model results must not depend on the split."""
import math
import os
import socket

import numpy as np
import pytest

from muscade_gpu import workloads as W
from muscade_gpu.shard import gather_to_root, my_share, shard_bounds


def test_shards_cover_every_item_once_and_balance_cost():
    rng = np.random.default_rng(0)
    for n, world in ((1, 1), (5, 2), (7, 8), (100, 3), (4096, 8)):
        costs = rng.integers(10, 400, n)
        b = shard_bounds(costs, world)
        assert len(b) == world and b[0][0] == 0 and b[-1][1] == n
        assert all(b[r][1] == b[r + 1][0] for r in range(world - 1))
        shares = [costs[lo:hi].sum() for lo, hi in b]
        assert max(shares) <= costs.sum() / world + costs.max()
    assert shard_bounds([], 3) == [(0, 0)] * 3


def _solve_models(params):
    from oracle import reference as REF

    out = []
    for p in params:
        m, _, times = W.build_batched([p])
        st = m.initialize()
        ref = REF.sweepx(m, st.dis, st, times[:3], OX=0, maxdx=1e-9, maxLl=math.inf)
        out.append(np.stack([X[0] for _, X in ref]))
    return out


def _worker(rank, world, port, params, result_path):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    costs = [p["nel"] for p in params]
    mine, idx = my_share(params, costs, rank, world)
    res = list(zip(idx.tolist(), _solve_models(mine)))
    allres = gather_to_root(res, dist)
    if rank == 0:
        flat = [r for part in allres for r in part]
        np.savez(result_path, idx=np.array([i for i, _ in flat]), *[x for _, x in flat])
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_run_gives_the_single_process_results(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    params = W.batched_params(6, nel_range=(10, 16), seed=3)
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    path = os.path.join(tmp_path, "res.npz")
    mp.start_processes(_worker, args=(2, port, params, path), nprocs=2, join=True, start_method="spawn")
    z = np.load(path)
    assert sorted(z["idx"].tolist()) == list(range(len(params)))
    single = _solve_models(params)
    for k, i in enumerate(z["idx"]):
        assert np.array_equal(z[f"arr_{k}"], single[i])
