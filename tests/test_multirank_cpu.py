"""The multi-GPU path of bench.py on the host: two gloo ranks (world_size 2),
each standing for one GPU.  Checks the rank environment, the barrier, the
max-over-ranks timing and the whole-job sum of voxel-steps that the bench line
reports (value = units all ranks processed / max time), for replicas and for a
population split across the ranks by robot (each rank stepping its own range
on the CPU oracle: the ranges cover the population once, and the per-robot
results equal those of the unsplit population)."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    r, w, local = bench.dist_env()
    dist = bench.init_dist(w)
    dist.barrier()
    # rank-dependent device time: the job time is the slowest rank's
    ms = 100.0 + 50.0 * r
    total_ms = bench.barrier_and_max(ms, w)
    voxels_per_rank, steps = 1000, 300
    value = voxels_per_rank * steps * w / (total_ms / 1e3)
    out[r] = (r, w, local, total_ms, value)
    dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_weak_scaling():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert sorted(out.keys()) == [0, 1]
    for r in range(2):
        rank, world, local, total_ms, value = out[r]
        assert (rank, world, local) == (r, 2, r)
        assert total_ms == 150.0  # the slower rank
        assert value == pytest.approx(1000 * 300 * 2 / 0.150)


def _shard_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    import oracle_bridge as ob
    from vx3g import workloads as wl
    r, w, _ = bench.dist_env()
    dist = bench.init_dist(w)
    robots = _population()
    lo, hi = wl.shard(len(robots), r, w)
    coms = []
    nv = 0
    for robot in robots[lo:hi]:
        s = ob.oracle_sim(robot)
        s.step(60)
        coms.append(s.com().tolist())
        nv += s.counts()[0]
    ranges = [None] * w
    dist.all_gather_object(ranges, (lo, hi))
    gathered = [None] * w
    dist.all_gather_object(gathered, coms)
    nv_job = bench.allreduce_sum(float(nv), w)
    out[r] = (ranges, [c for part in gathered for c in part], nv_job)
    dist.destroy_process_group()


def _population():
    import numpy as np
    from vx3g import workloads as wl
    rng = np.random.default_rng(4)
    mats = [wl.Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, cte=0.01) for _ in range(2)]
    return [wl.bernoulli_body(rng, tuple(int(x) for x in rng.integers(2, 5, size=3)), 0.8, mats, random_phase=True,
                              temp_vary=True, temp_amplitude=20.0) for _ in range(5)]


def test_shard_ranges_cover_the_population_once():
    from vx3g import workloads as wl
    for n in (0, 1, 5, 7, 1024):
        for world in (1, 2, 3, 8):
            ranges = [wl.shard(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [hi - lo for lo, hi in ranges]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_split_a_population_by_robot():
    import numpy as np
    import oracle_bridge as ob
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_shard_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    robots = _population()
    whole, nv = [], 0
    for robot in robots:
        s = ob.oracle_sim(robot)
        s.step(60)
        whole.append(s.com().tolist())
        nv += s.counts()[0]
    for r in range(2):
        ranges, coms, nv_job = out[r]
        assert ranges == [(0, 3), (3, 5)]
        assert np.array_equal(np.array(coms), np.array(whole))  # independent robots: identical per robot
        assert nv_job == nv
