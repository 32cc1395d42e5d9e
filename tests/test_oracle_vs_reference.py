"""The oracle against the reference's own VX3 physics compiled on the host
(oracle/_ref, built from the reference sources by oracle/Makefile), on seeded
random robots that combine every feature the oracle restates -- thermal
actuation, self-collision, detach, material removal, cilia, force fields -- and
over the settings the fixed workloads leave at their defaults (densities, Poisson's
ratios, isMeasured, thermal delays, Fixed voxels, lattice size, DtFrac, damping,
gravity, static temperature) and over the run-time features together (signals,
boundary conditions, attachment, detach) and the stress-strain models together (bilinear
with plastic unloading, data-point curves, failure, Poisson's ratio), compared bit for bit: positions, orientations,
momenta, temperatures, contact forces, surface sets, time and centre of mass.  Skipped where the reference build is absent."""

import numpy as np
import pytest

import feature_mix
import oracle_bridge as ob

pytestmark = pytest.mark.skipif(not ob.ref_available(), reason="reference host build (oracle/_ref) not present")


@pytest.mark.parametrize("gen,seed", [("robot", s) for s in range(8)] + [("robot_settings", s) for s in range(8)]
                         + [("robot_dynamic", s) for s in range(8)] + [("robot_models", s) for s in range(8)])
def test_oracle_matches_reference_build(gen, seed):
    robot = getattr(feature_mix, gen)(seed)
    a, b = ob.ref_sim(robot), ob.oracle_sim(robot)
    assert a.counts()[:2] == b.counts()[:2]
    for _ in range(4):
        na, nb = a.step(60), b.step(60)
        assert na == nb
        va, vb = a.voxels(), b.voxels()
        for key in ("pos", "orient", "linmom", "angmom", "tempe"):
            assert np.array_equal(va[key], vb[key]), key
        assert np.array_equal(a.surface(), b.surface())
        assert np.array_equal(a.last_contact(), b.last_contact())
        assert a.time() == b.time()
        assert np.array_equal(a.com(), b.com())  # over the measured voxels
