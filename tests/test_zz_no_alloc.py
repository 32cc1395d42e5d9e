"""vx3g_recommended_dt_noalloc (stable time step with module-static scratch)
against the time step vx3g_create computes with its own scratch.

vx3g_create sets dt = (float)(DtFrac * max(recommendedTimeStep, 1e-10)); at step
0 (no strain yet) the no-allocation entry point must give the same
recommendedTimeStep, so the float dt it implies must equal vx3g_dt bit for bit, on
two calls in a row.  Covers palettes with Poisson's ratio off and on (the
strain-dependent stiffness branch), FP64 and mixed-precision contexts, several
robots, a deformed state against the oracle, and the 4096-robot limit."""

import numpy as np
import pytest

from vx3g import abi
from vx3g import workloads as wl

pytestmark = pytest.mark.gpu


def _robots():
    rng = np.random.default_rng(11)
    out = []
    for i in range(6):
        mats = [wl.Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, rho=float(rng.uniform(500, 2000)))
                for _ in range(3)]
        out.append(wl.bernoulli_body(rng, tuple(int(x) for x in rng.integers(3, 9, 3)), 0.8, mats,
                                     volume_effects=bool(i % 2), dt_frac=float(rng.uniform(0.3, 0.95))))
    return out


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_noalloc_dt_matches_create_time_dt(precision):
    robots = _robots()
    b = abi.Batch(robots, precision)
    ref = np.asarray(b.dt(), np.float32)
    frac = np.array([r.dt_frac for r in robots])
    for _ in range(2):
        rdt = b.recommended_dt_noalloc()
        got = (frac * np.maximum(rdt, 1e-10)).astype(np.float32)
        assert np.array_equal(got, ref), (got, ref)
    b.close()


@pytest.mark.parametrize("precision,tol", [(abi.PRECISION_FP64, 1e-12), (abi.PRECISION_MIXED, 1e-6)])
def test_noalloc_dt_follows_the_deformed_state(precision, tol):
    """After 300 steps of falling and landing, the links are strained: the
    strain-dependent stiffness branch (Poisson's ratio on) moves the stable step
    away from its step-0 value.  Against the oracle's recommendedTimeStep on its own
    run of the same robots (creation-time transverse area, current strain and rest
    length), on two calls in a row."""
    import oracle_bridge as ob
    robots = _robots()
    b = abi.Batch(robots, precision)
    step0 = b.recommended_dt_noalloc()
    b.step(300)
    sims = [ob.oracle_sim(r) for r in robots]
    for s in sims:
        s.step(300)
    ref = np.array([s.recommended_dt() for s in sims])
    for _ in range(2):
        got = b.recommended_dt_noalloc()
        assert np.allclose(got, ref, rtol=tol, atol=0), (got, ref)
    moved = np.abs(ref / step0 - 1)
    assert np.all(moved[[bool(r.volume_effects) for r in robots]] > 1e-9)  # the strain branch is exercised
    b.close()


def test_noalloc_dt_rejects_more_than_4096_robots():
    one = wl.Robot(grid=np.ones((1, 1, 1), np.uint8), materials=[wl.Material()], floor=False)
    b = abi.Batch([one] * 4097, abi.PRECISION_FP64)
    with pytest.raises(abi.Vx3gError, match="4096"):
        b.recommended_dt_noalloc()
    b.close()
