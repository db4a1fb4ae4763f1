"""Host logic of the batched sweep across ranks: a world_size-2 gloo job
splits the instances, each rank "solves" its share (a stand-in cost), and the
gathered costs come back complete and in instance order on every rank."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from magudi_gb300 import sweep


def test_cases_are_seeded_and_cycle_amplitudes():
    a, b = sweep.cases(64), sweep.cases(64)
    assert a == b
    assert {n for n, _ in a} <= set(sweep.SIZES)
    assert [amp for _, amp in a[:20]] == [10.0 ** (-2.0 - 0.25 * k) for k in range(20)]
    assert a[20][1] == a[0][1]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shard_partitions_and_balances(world):
    cs = sweep.cases(64)
    parts = [sweep.shard(cs, r, world) for r in range(world)]
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(64))
    loads = [sum(cs[i][0] ** 2 for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(n * n for n in sweep.SIZES)


def test_fd_error_rows():
    rows = sweep.fd_errors(1.0, 2.0, [0.1, 0.01], [1.2, 1.02])
    assert np.allclose([r[2] for r in rows], [2.0, 2.0])
    assert max(r[3] for r in rows) < 1e-12


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cs = sweep.cases(64)
    mine = sweep.shard(cs, rank, world)
    costs = [cs[i][0] * 1e-3 + cs[i][1] for i in mine]  # stand-in for each instance's J
    allc = sweep.gather_costs(mine, costs, len(cs))
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), allc)
    dist.barrier()
    dist.destroy_process_group()


def test_gather_over_two_gloo_ranks(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    cs = sweep.cases(64)
    expect = np.array([n * 1e-3 + a for n, a in cs])
    for r in range(world):
        got = np.load(tmp_path / f"rank{r}.npy")
        assert np.array_equal(got, expect)


SMALL = {129: 25, 161: 27, 201: 29, 257: 31, 321: 33, 385: 35}


def _instance_cost(n, amplitude):
    """J of one sweep instance on a small grid standing in for its size: the
    monopole forward run with the control forcing amplitude x a fixed
    seeded direction, on the strict CPU oracle."""
    import oracle_lib
    from helpers import small_monopole
    P = small_monopole(n=SMALL[n], ny=SMALL[n], n_steps=4, save_interval=2, controller_switch=True)
    o = oracle_lib.Oracle(P)
    rng = np.random.default_rng(n)
    o.set_control_forcing(amplitude * rng.standard_normal((16, o.actuator_points())))
    return o.run_forward(4, 2, keep_stages=False)


def _oracle_rank_main(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cs = sweep.cases(10)
    mine = sweep.shard(cs, rank, world)
    costs = [_instance_cost(*cs[i]) for i in mine]
    allc = sweep.gather_costs(mine, costs, len(cs))
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), allc)
    np.save(os.path.join(out_dir, f"mine{rank}.npy"), np.array(mine))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_sweep_of_real_instances_over_two_gloo_ranks(tmp_path):
    """Each rank runs the real forward solves of its shard (the oracle, on
    small grids); the gathered costs equal a serial pass over all cases, bit
    for bit, and the shards are disjoint."""
    world = 2
    mp.spawn(_oracle_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    cs = sweep.cases(10)
    serial = np.array([_instance_cost(n, a) for n, a in cs])
    shards = [set(np.load(tmp_path / f"mine{r}.npy").tolist()) for r in range(world)]
    assert not (shards[0] & shards[1]) and (shards[0] | shards[1]) == set(range(len(cs)))
    for r in range(world):
        assert np.array_equal(np.load(tmp_path / f"rank{r}.npy"), serial)
