"""The oracle continues a run taken elsewhere (vxo_set_voxels + vxo_set_run_state):
an oracle run stopped after N steps and its whole state loaded into a fresh oracle of
the same robot give bit-identical continuations.  This is what lets a GPU run be
continued on the CPU oracle from any step (the full-size parity test)."""

import numpy as np

import feature_mix
import oracle_bridge as ob


def test_oracle_continues_a_loaded_run_bit_for_bit():
    for seed in (0, 2, 5):
        robot = feature_mix.robot(seed)
        if robot.enable_detach or robot.secondary_experiment:
            continue  # the link table's changes are not part of the loaded state
        a = ob.oracle_sim(robot)
        a.step(120)
        v, lk, t = a.voxels(), a.links(), a.topology()
        flags = (t["small"] & 1) | np.where(t["states"] & 1, 4, 0)
        b = ob.oracle_sim(robot)
        b.set_state(v["pos"], v["orient"], v["linmom"], v["angmom"], a.time(), v["tempe"], v["flags"] & 8,
                    lk["local9"], lk["strain"], lk["maxstrain"], flags)
        a.step(80)
        b.step(80)
        va, vb = a.voxels(), b.voxels()
        for k in ("pos", "orient", "linmom", "angmom", "tempe", "flags"):
            assert np.array_equal(va[k], vb[k]), (seed, k)
        assert np.array_equal(a.last_contact(), b.last_contact())
        assert a.time() == b.time()
