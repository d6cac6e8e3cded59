"""Multi-rank sweeps on CPU: the partition of (variant, frequency) points and
the gather to rank 0, with world_size-2 gloo process groups (no GPU)."""

import os
import socket

import numpy as np
import pytest

from mom25d_gb300.shard import partition, point_cost, sharded_map


def test_partition_covers_every_item_once():
    rng = np.random.default_rng(0)
    costs = rng.uniform(1, 10, 37)
    for world in (1, 2, 3, 8):
        parts = partition(costs, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        assert all(p == sorted(p) for p in parts)


def test_partition_balances_variants_by_lu_cost():
    # 16 bandpass-like variants, N 1.5k-5k, 128 frequencies each: LPT keeps
    # the heaviest rank within one point of the mean load
    rng = np.random.default_rng(1)
    n = rng.integers(1500, 5000, 16)
    costs = np.repeat([point_cost(v) for v in n], 8)
    parts = partition(costs, 4)
    loads = np.array([costs[p].sum() for p in parts])
    assert loads.max() - loads.mean() <= costs.max()


def test_partition_is_deterministic_and_rejects_bad_world():
    c = [3, 1, 2, 3, 1]
    assert partition(c, 2) == partition(c, 2) == [[0, 2], [1, 3, 4]]
    with pytest.raises(ValueError):
        partition(c, 0)


def _fake_point(f):
    # stands in for Solver.point: a deterministic 2-port result of f
    S = np.array([[np.exp(-1j * f), 0.1 * f], [0.1 * f, np.exp(-2j * f)]])
    return S, f * 1e-9


def _rank_main(rank, world, port, items, costs, out_path):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = sharded_map(items, costs, _fake_point, rank, world)
        if rank == 0:
            np.save(out_path, np.array([r[0] for r in res]))
        else:
            assert res is None
    finally:
        dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_sharded_map_two_gloo_ranks_matches_one_process(tmp_path):
    import torch.multiprocessing as mp

    items = list(np.linspace(0.5e9, 8e9, 11))
    costs = [point_cost(5943)] * len(items)
    out = str(tmp_path / "S.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), items, costs, out), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(out)
    want = np.array([_fake_point(f)[0] for f in items])
    np.testing.assert_array_equal(got, want)
