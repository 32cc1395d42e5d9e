"""The C restatement (oracle/vx3_oracle.c) against the reference's own step.

Golden vectors come from the reference sources compiled on the host
(tests/golden/make_golden.py).  The restatement must reproduce them bit for
bit: same topology and ordering, same derived material constants, and the
same voxel/link state after every snapshot interval (with attachment: the same
runtime links, in the same order, on the same faces).
"""

import numpy as np
import pytest

import golden_cases
import oracle_bridge as ob

CASES = golden_cases.names()


@pytest.mark.parametrize("name", CASES)
def test_topology_and_materials(name):
    robot, d = golden_cases.load(name)
    s = ob.oracle_sim(robot)
    t = s.topology()
    for k in ("mat", "ijk", "slots", "negpos", "axis"):
        assert np.array_equal(t[k], d["topo_" + k]), k
    m = s.materials(len(robot.materials))
    for k in ("vmat", "nomsize", "fixed_measured", "lmat", "lmat_of_link"):
        assert np.array_equal(m[k], d["mat_" + k]), k
    assert s.recommended_dt() == d["recommended_dt0"][0]
    if "link_curves" in d.files:  # non-linear link materials: the merged stress-strain points
        got = s.link_curves()
        assert np.array_equal(np.array([len(c) for c in got], np.int32), d["link_curve_n"])
        assert np.array_equal(np.concatenate(got), d["link_curves"])


@pytest.mark.parametrize("name", CASES)
def test_trajectory_bit_exact(name):
    robot, d = golden_cases.load(name)
    s = ob.oracle_sim(robot)
    done = 0
    for snap in d["snap_steps"]:
        s.step(int(snap) - done)
        done = int(snap)
        v, lk, t = s.voxels(), s.links(), s.topology()
        got = dict(pos=v["pos"], orient=v["orient"], linmom=v["linmom"], angmom=v["angmom"], tempe=v["tempe"],
                   flags=v["flags"], strain=lk["strain"], maxstrain=lk["maxstrain"], rest=lk["rest"],
                   local9=lk["local9"], forces=lk["forces"], contact=s.last_contact(), com=s.com(),
                   small=t["small"], states=t["states"], surface=s.surface())
        # (a link with a Fixed end carries NaN in that end's force: the fixed voxel never steps, so its
        # dampingMultiplier divides by a previousDt of 0; the fixed voxel never reads it)
        if f"s{snap}_soffset" in d.files:
            got["soffset"] = s.link_offsets()
        if f"s{snap}_signal" in d.files:
            got["signal"] = s.signals()
        if f"s{snap}_negpos" in d.files:  # attachment: the link table with its runtime links
            got.update(negpos=t["negpos"], axis=t["axis"], slots=t["slots"],
                       lmat_of_link=s.materials(len(robot.materials))["lmat_of_link"])
        for k, a in got.items():
            b = d[f"s{snap}_{k}"]
            assert np.array_equal(a, b, equal_nan=True), f"{name} step {snap}: {k} differs (max {np.max(np.abs(a - b)) if a.shape == b.shape else 'shape'})"
        assert s.time() == d[f"s{snap}_time"][0]
        assert np.float32(s.dt()) == d[f"s{snap}_dt"][0]
