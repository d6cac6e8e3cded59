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


class _StubSolver:
    """Stands in for Solver on a CPU rank (there is no CPU path of the
    engine): point(f) returns a deterministic 2-port result of f and of the
    lumped value override "Z1", so the test sees whether values reached every
    rank."""

    class _Port:
        def __init__(self, name):
            self.name = name

    def __init__(self, stale=None):
        import types

        self.mesh = types.SimpleNamespace(n_unknowns=1500)
        self.values = dict(stale or {})
        self.ports = [self._Port("P1"), self._Port("P2")]

    def point(self, f, keep_currents=False):
        r = float(self.values.get("Z1", 0.0))
        g = f * 1e-9
        S = np.array([[np.exp(-1j * g), 0.1 + r], [0.1 + r, np.exp(-2j * g)]])
        z0 = np.array([50.0, 50.0 + r])
        return (S, z0, 1j * g * np.ones(2), z0.astype(complex), np.array([1e-3, 2e-3]) * g, None,
                dict(refine_steps=int(g) % 5, waves=np.eye(2) * g))


def _sweep_rank_main(rank, world, port, freqs, values, out_path):
    import torch.distributed as dist

    from mom25d_gb300.shard import sweep_sharded

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        res = sweep_sharded(_StubSolver(stale={"Z1": 7.0}), freqs, rank, world, values=values)
        if rank == 0:
            np.savez(out_path, S=res.S, z0=res.z0, gamma=res.gamma, z0_line=res.z0_line, res=res.fit_residual,
                     waves=res.waves, steps=np.array(res.info["refine_steps"]), ranks=res.info["ranks"],
                     names=np.array(res.port_names), freqs=res.freqs)
        else:
            assert res is None
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("values", [None, {"Z1": 2.0}])
def test_sweep_sharded_assembles_the_full_result(tmp_path, values):
    """sweep_sharded on two gloo ranks: rank 0 gets every frequency's S, z0,
    gamma, z0_line, residual, waves and refine steps in frequency order, as a
    one-process sweep_sharded gives them, and the value overrides (or their
    absence, which clears a stale override) reach both ranks."""
    import torch.multiprocessing as mp

    from mom25d_gb300.shard import sweep_sharded

    freqs = np.linspace(1e9, 12e9, 9)
    out = str(tmp_path / "r.npz")
    mp.start_processes(_sweep_rank_main, args=(2, _free_port(), freqs, values, out), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(out)
    want = sweep_sharded(_StubSolver(stale={"Z1": 7.0}), freqs, values=values)
    np.testing.assert_array_equal(got["freqs"], freqs)
    for k, v in (("S", want.S), ("z0", want.z0), ("gamma", want.gamma), ("z0_line", want.z0_line),
                 ("res", want.fit_residual), ("waves", want.waves)):
        np.testing.assert_array_equal(got[k], v, err_msg=k)
    assert list(got["steps"]) == want.info["refine_steps"]
    assert int(got["ranks"]) == 2
    assert list(got["names"]) == ["P1", "P2"]
    r = 0.0 if values is None else values["Z1"]
    assert np.all(got["S"][:, 0, 1] == 0.1 + r)


def test_batch_point_order_is_longest_first():
    """Batched variants hand out their points largest N first (the LPT rule
    on the N^3 cost), each variant's frequencies in order."""
    from mom25d_gb300.batch import point_order

    order = point_order([1524, 4972, 3064], [2, 3, 1])
    assert order == [(1, 0), (1, 1), (1, 2), (2, 0), (0, 0), (0, 1)]


def test_tuning_table_rows_by_size(tmp_path):
    """A tuning table picks the first row whose n_max covers N (the last one
    beyond) and round-trips through its JSON file."""
    import json

    from mom25d_gb300.autotune import Tuning, load_table

    rows = [dict(n_max=None, panel_cluster_min=16, wave_ctas=0, tc_chunk=1),
            dict(n_max=2000, panel_cluster_min=4, wave_ctas=16, tc_chunk=2)]
    p = tmp_path / "t.json"
    p.write_text(json.dumps(dict(rows=rows)))
    t = load_table(str(p))
    assert t.knobs(1500) == (4, 16, 2, 0)
    assert t.knobs(2000) == (4, 16, 2, 0)
    assert t.knobs(9000) == (16, 0, 1, 0)
    assert Tuning.fixed(tc_chunk=2).knobs(10 ** 6) == (0, 0, 2, 0)
    assert Tuning.fixed(tc_tile_n=128).knobs(1) == (0, 0, 0, 128)
    with pytest.raises(ValueError):
        Tuning([dict(n_max=1)])


def test_sweep_tuning_choice():
    """A mixed-precision sweep takes the measured table (by N) unless the
    solver's tuning says otherwise; fp64 sweeps keep the process defaults."""
    from mom25d_gb300.autotune import Tuning, load_table
    from mom25d_gb300.solver import Solver

    s = object.__new__(Solver)
    s.precision, s.tuning = "mixed", "table"
    t = s._sweep_tuning()
    assert t is not None and t.knobs(5943) == load_table().knobs(5943)
    s.tuning = fixed = Tuning.fixed(panel_cluster_min=8)
    assert s._sweep_tuning() is fixed
    s.tuning = None
    assert s._sweep_tuning() is None
    s.precision, s.tuning = "fp64", "table"
    assert s._sweep_tuning() is None
    s.precision, s.tuning = "mixed", "best"
    with pytest.raises(ValueError):
        s._sweep_tuning()


def test_sweep_workers_take_current_settings():
    """A worker made by an earlier sweep takes the solver's settings as they
    are now (a learned remainder or tuning attached between sweeps)."""
    import threading
    from types import SimpleNamespace

    from mom25d_gb300.solver import Solver

    s = object.__new__(Solver)
    s._blocks_host = True
    s._sib_lock = threading.Lock()
    s._siblings = [SimpleNamespace(**{k: None for k in Solver._SETTINGS})]
    for k in Solver._SETTINGS:
        setattr(s, k, "now-" + k)
    sib = s._sibling(1)
    assert all(getattr(sib, k) == "now-" + k for k in Solver._SETTINGS)
    assert s._sibling(0) is s
