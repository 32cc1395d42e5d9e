"""The mixed-precision step against the FP64 step over whole populations: the
1024-robot batch ([4,16]^3, Bernoulli(0.7), floor) and the 256-robot batch with
self-collision ([8,20]^3, Bernoulli(0.65)), 2000 steps each.

The bar is the relative centre-of-mass error |COM_mixed - COM_fp64| / |COM_fp64|
<= 1e-5.  Walking robots with floor friction are chaotic: a stick/slip decision
taken one step apart diverges the trajectories.  So besides the distribution of
the mixed error, the FP64 step is run once more from positions nudged by +-1e-9 m
(far below an FP32 rounding of a position), and the mixed error must stay within
the spread that this perturbation alone produces in the FP64 step."""

import numpy as np
import pytest

from vx3g import abi
from vx3g import workloads as wl

pytestmark = pytest.mark.gpu

STEPS = 2000


def _rel(a, b):
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


def _com_after(robots, precision, nudge=0.0):
    b = abi.Batch(robots, precision)
    if nudge:
        st = b.state()
        st["pos"] += nudge * np.random.default_rng(1).choice([-1.0, 1.0], size=st["pos"].shape)
        b.set_state(**st)
    b.step(STEPS)
    c, s = b.com(), b.status()
    b.close()
    assert np.all(s == 0)
    return c


@pytest.mark.parametrize("name", ["c3", "c5"])
def test_population_mixed_com_error(name):
    robots = wl.c3_population() if name == "c3" else wl.c5_population_collisions()
    c64 = _com_after(robots, abi.PRECISION_FP64)
    err = _rel(_com_after(robots, abi.PRECISION_MIXED), c64)
    floor = _rel(_com_after(robots, abi.PRECISION_FP64, nudge=1e-9), c64)
    # the distribution: almost every robot far inside the bar
    assert np.median(err) <= 1e-7, np.median(err)
    assert np.percentile(err, 90) <= 1e-6, np.percentile(err, 90)
    assert np.mean(err <= 1e-5) >= 0.99, np.sort(err)[-8:]
    # the tail: no worse than what a 1e-9 m perturbation does to the FP64 step itself
    assert err.max() <= max(1e-5, 3 * floor.max()), (err.max(), floor.max())
