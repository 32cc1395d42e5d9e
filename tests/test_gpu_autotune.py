"""Launch-shape autotuning (vx3g_autotune): every compiled shape of the mixed
passes gives bit-identical states, the tuner advances exactly like vx3g_step,
and the JSON cache round-trips."""

import json

import numpy as np
import pytest

from vx3g import abi
from vx3g import workloads as wl

pytestmark = pytest.mark.gpu

# the compiled shapes, (threads per block, minimum resident blocks), in index order
LINK_SHAPES = [[256, 1], [256, 4], [128, 9], [128, 10], [64, 20], [256, 5]]
VOXEL_SHAPES = [[256, 1], [256, 3], [128, 7], [128, 8], [64, 14], [64, 16]]


def _robots():
    return wl.c3_population(seed=5)[:48]


def _state(b):
    s = b.state()
    return np.concatenate([s[k].reshape(-1) for k in ("pos", "orient", "linmom", "angmom")])


def test_every_shape_gives_identical_states(tmp_path):
    robots = _robots()
    ref = abi.Batch(robots, abi.PRECISION_MIXED)
    ref.step(150)
    want = _state(ref)
    key = None
    for k in range(len(LINK_SHAPES)):
        b = abi.Batch(robots, abi.PRECISION_MIXED)
        if key is None:  # learn the cache key from a tuning run
            path = tmp_path / "probe.json"
            b.autotune(150, path)
            key = next(iter(json.loads(path.read_text())))
        else:
            path = tmp_path / f"shape{k}.json"
            path.write_text(json.dumps({key: [k, k]}))
            b.autotune(150, path)
            assert list(b.launch_shapes()) == LINK_SHAPES[k] + VOXEL_SHAPES[k]
        assert b.steps_taken() == 150
        assert np.array_equal(_state(b), want), k


def test_cached_choice_is_applied(tmp_path):
    robots = _robots()
    b = abi.Batch(robots, abi.PRECISION_MIXED)
    path = tmp_path / "cache.json"
    b.autotune(64, path)
    chosen = b.launch_shapes().copy()
    entry = json.loads(path.read_text())
    assert len(entry) == 1
    c = abi.Batch(robots, abi.PRECISION_MIXED)
    c.autotune(10, path)  # cached: no timing, same shapes
    assert np.array_equal(c.launch_shapes(), chosen)
    assert c.steps_taken() == 10


def test_fork_points_give_identical_states(tmp_path):
    """The overlapped mixed step forks its side stream after the rebuild kernel or
    before the displacement check (vx3g_autotune picks one): the states are identical,
    in graphs and in single steps, and the tuner's choice lands in the cache."""
    rng = np.random.default_rng(8)
    mats = [wl.Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, cte=0.01) for _ in range(3)]
    robots = [wl.bernoulli_body(rng, tuple(int(x) for x in rng.integers(6, 11, size=3)), 0.7, mats,
                                random_phase=True, temp_vary=True, temp_amplitude=39.0, enable_collision=True,
                                z_offset=1) for _ in range(5)]
    probe = tmp_path / "probe.json"
    t = abi.Batch(robots, abi.PRECISION_MIXED)
    t.autotune(64, probe)  # shapes, then whole steps at both fork points
    assert t.steps_taken() == 64
    key, entry = next(iter(json.loads(probe.read_text()).items()))
    assert len(entry) == 3 and entry[2] in (0, 1)
    states = []
    for fk in (0, 1):
        path = tmp_path / f"fork{fk}.json"
        path.write_text(json.dumps({key: [entry[0], entry[1], fk]}))
        b = abi.Batch(robots, abi.PRECISION_MIXED)
        b.autotune(0, path)
        b.step(200)  # graph chunks
        b.step(7)    # single steps
        assert np.all(b.status() == 0)
        states.append(_state(b))
    assert np.array_equal(states[0], states[1])
