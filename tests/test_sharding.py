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


def test_riser_subset_is_a_slice_of_the_whole_set():
    """bench.py's riser shards: risers(n, subset=(lo, hi)) builds risers lo..hi-1
    of the seeded set of n, with their own prescribed motions."""
    full, _ = W.risers(nriser=6, nel=4)
    part, _ = W.risers(nriser=6, nel=4, subset=(2, 5))
    nn = 5  # nodes per riser
    assert part.nnod == 3 * nn
    for k in range(3):
        for j in range(nn):
            assert np.array_equal(part.coord(1 + k * nn + j), full.coord(1 + (k + 2) * nn + j))
    from muscade_gpu.elements import group_time_values

    gf = next(g for g in full.groups if g.key[0] == "DofConstraint" and g.key[-1] == "surge")
    gp = next(g for g in part.groups if g.key[0] == "DofConstraint" and g.key[-1] == "surge")
    for t in (1.0, 7.5, 12.0):
        assert np.array_equal(group_time_values(gp, "offset", t), group_time_values(gf, "offset", t)[2:5])


def _device_worker(rank, world, port, params, result_path):
    import torch.distributed as dist

    from muscade_gpu.device import DeviceModel

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    mine, idx = my_share(params, [p["nel"] for p in params], rank, world)
    res = []
    if len(mine):
        m, offs, times = W.build_batched(mine)
        st = m.initialize()
        dm = DeviceModel(m, st.dis, device=0)
        rc, x, _ = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-9, maxLl=math.inf, per_component=True)
        dm.close()
        assert rc == 0
        bounds = list(offs) + [m.nnod]
        for k, i in enumerate(idx):
            d = W.node_dofs(m, np.arange(bounds[k] + 1, bounds[k + 1] + 1))
            res.append((int(i), x[:, 0, d[d >= 0]]))
    allres = gather_to_root(res, dist)
    if rank == 0:
        flat = [r for part in allres for r in part]
        np.savez(result_path, idx=np.array([i for i, _ in flat]), *[x for _, x in flat])
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.gpu
def test_two_rank_device_run_gives_the_single_process_results(tmp_path):
    """The same split on the device path: two gloo ranks on one GPU, each
    solving its share of the models in one context (per-model convergence);
    every model's states equal, bitwise, those of one process solving all."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from muscade_gpu import _lib
    from muscade_gpu.device import DeviceModel

    _lib.build()
    params = W.batched_params(8, nel_range=(10, 30), seed=5)
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    path = os.path.join(tmp_path, "res.npz")
    mp.start_processes(_device_worker, args=(2, port, params, path), nprocs=2, join=True, start_method="spawn")
    z = np.load(path)
    assert sorted(z["idx"].tolist()) == list(range(len(params)))
    m, offs, times = W.build_batched(params)
    st = m.initialize()
    dm = DeviceModel(m, st.dis, device=0)
    rc, x, _ = dm.sweepx(0, times, st.time, list(st.X), maxdx=1e-9, maxLl=math.inf, per_component=True)
    dm.close()
    assert rc == 0
    bounds = list(offs) + [m.nnod]
    for k, i in enumerate(z["idx"]):
        d = W.node_dofs(m, np.arange(bounds[i] + 1, bounds[i + 1] + 1))
        assert np.array_equal(z[f"arr_{k}"], x[:, 0, d[d >= 0]]), i
