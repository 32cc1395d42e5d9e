"""Fault path of the collision list rebuild, driven without faulting the GPU.

The rebuild of a large robot's contact lists runs phases separated by grid
barriers; each wait is bounded, and a wait that runs out sets the device error
word and returns.  The test hook vx3g_debug_barrier pre-counts arrivals that
never happen and lowers the poll limit, so every wait runs out within
microseconds: the step must finish, vx3g_status must report VX3G_ERR_DEVICE,
and after the report the context must recover -- the barrier words cleared,
every list rebuilt -- and follow a clean run of the same robot bit for bit
(the lists are supersets of the pairs in reach, so skipping one rebuild while
no voxel has moved far changes no contact force)."""

import numpy as np
import pytest

from vx3g import abi
from vx3g import workloads as wl

pytestmark = pytest.mark.gpu


def _large_robot():
    # more than 6144 collision-surface voxels: its lists are built on the global
    # hashed grid, the phase with the grid barriers
    rng = np.random.default_rng(5)
    mats = [wl.Material(E=1e6, nu=0.35), wl.Material(E=1e6, nu=0.35, cte=0.01)]
    return wl.bernoulli_body(rng, (26, 26, 26), 0.6, mats, temp_vary=True, temp_amplitude=39.0,
                             enable_collision=True, enable_expansion=1)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_barrier_timeout_is_reported_and_recovered(precision):
    r = _large_robot()
    clean = abi.Batch([r], precision)
    b = abi.Batch([r], precision)
    assert b.ns > 6144
    clean.step(40)
    b.step(10)
    assert np.all(b.status() == 0)
    b.debug_barrier(polls=256, arrivals=1 << 30)  # every wait of the next rebuild runs out
    b.step(5)  # the first step's rebuild gives up; the next ones are skipped until reported
    b.synchronize()
    with pytest.raises(abi.Vx3gError, match="grid barrier"):
        b.status()
    b.debug_barrier(polls=0, arrivals=0)  # back to the default limit
    b.step(25)
    assert np.all(b.status() == 0)  # recovered: no further error
    got, ref = b.state(), clean.state()
    for k in ("pos", "orient", "linmom", "angmom"):
        assert np.array_equal(got[k], ref[k]), k
    assert np.array_equal(b.voxel_aux()["contact"], clean.voxel_aux()["contact"])
    b.close()
    clean.close()
