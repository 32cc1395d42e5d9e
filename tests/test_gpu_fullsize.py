"""The full-size single body -- 64^3 Bernoulli(0.6), two materials, 39 C / 5 Hz
actuation, self-collision and floor, the configuration the benchmark runs -- against
the oracle in its contact-heavy regime.

From ~4,000 steps on the thermally contracted body is folded into heavy self-contact
(around step 5,000 about 100,000 voxels feel a contact force; Verlet-list rebuilds every few steps
on the global hashed grid).  The FP64 kernels run there from step 0; their whole
state (voxel state, time, temperatures, static friction, link state) is then loaded
into the oracle, and both continue: the oracle with the reference's all-pairs
surface loop (S(S-1)/2 = 1.1e10 pairs per step, on every host core, summed in the
serial loop's order).  Per step: positions within 1e-6 voxel sizes, the same set of
voxels in contact, contact forces equal to 1e-9 relative.  A pair missing from a
candidate list would show up as a missing or smaller contact force."""

import os

import numpy as np
import pytest

import oracle_bridge as ob
from vx3g import abi
from vx3g import workloads as wl

pytestmark = pytest.mark.gpu

START, STEPS = 4700, 8


def test_contact_heavy_64cube_fp64_matches_oracle_all_pairs():
    robot = wl.c2_single_body()[0]
    b = abi.Batch([robot], abi.PRECISION_FP64)
    b.step(START)
    st, aux, lk = b.state(), b.voxel_aux(), b.links()
    o = ob.oracle_sim(robot)
    o.set_exact_threads(os.cpu_count() or 1)
    o.set_state(st["pos"], st["orient"], st["linmom"], st["angmom"], b.time()[0], aux["tempe"], aux["flags"] & 8,
                lk["local9"], lk["strain"], lk["maxstrain"], lk["small"])
    assert np.float32(b.dt()[0]) == np.float32(o.dt())  # the same step length
    touching = []
    for k in range(STEPS):
        b.step(1)
        o.step(1)
        got, ref = b.state()["pos"], o.voxels()["pos"]
        err = np.max(np.abs(got - ref))
        assert err <= 1e-6 * robot.vox_size, f"step {START + k + 1}: position error {err:.3e} m"
        cg, cr = b.voxel_aux()["contact"], o.last_contact()
        on_g, on_r = np.abs(cg).sum(1) > 0, np.abs(cr).sum(1) > 0
        assert np.array_equal(on_g, on_r), f"step {START + k + 1}: contact sets differ"
        np.testing.assert_allclose(cg, cr, rtol=1e-9, atol=1e-9 * np.abs(cr).max())
        touching.append(int(on_r.sum()))
    assert min(touching) > 20000, touching  # the contact-heavy regime indeed
    assert np.all(b.status() == 0)
