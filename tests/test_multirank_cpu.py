"""The multi-GPU path of bench.py on the host: two gloo ranks (world_size 2),
each standing for one GPU running its own replica of the workload.  Checks the
rank environment, the barrier, the max-over-ranks timing and the whole-job sum
of voxel-steps that the bench line reports (weak scaling: value = units all ranks
processed / max time)."""

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
