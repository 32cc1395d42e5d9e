"""The VX3_SimulationManager drop-in (vx3g_sim runner) on the GPU: a base VXA plus
VXD overrides in a directory, run to the StopConditionFormula, report XML
compared with the CPU oracle running the same merged robots."""

import os
import subprocess
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import oracle_bridge as ob
from vx3g import build as vbuild
from vx3g import workloads as wl

pytestmark = pytest.mark.gpu


def _oracle_until(robot, stop_time):
    s = ob.oracle_sim(robot)
    c0 = s.com()
    steps = 0
    while not (s.time() - stop_time > 0):  # CUDA_Simulation: StopConditionMet() checked before every step
        s.step(1)
        steps += 1
    return s, c0, steps


def test_runner_merges_vxd_and_matches_oracle(tmp_path):
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    rng = np.random.default_rng(3)
    mats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=3e5, nu=0.35, cte=0.0)]
    base = wl.bernoulli_body(rng, (5, 4, 3), 0.8, mats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                             stop_time=0.02, fitness_x=True)
    other = wl.bernoulli_body(rng, (6, 3, 4), 0.8, mats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                              stop_time=0.02, fitness_x=True)
    (tmp_path / "base.vxa").write_text(wl.to_vxa(base))
    (tmp_path / "a_same.vxd").write_text("<VXD>\n</VXD>\n")
    (tmp_path / "b_other.vxd").write_text(wl.to_vxd(other))
    out = tmp_path / "report.xml"
    r = subprocess.run([exe, "-i", str(tmp_path), "-o", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rep = ET.parse(out).getroot()
    for name, robot in (("a_same", base), ("b_other", other)):
        node = rep.find(f"detail/{name}")
        assert node is not None, name
        s, c0, _ = _oracle_until(robot, 0.02)
        assert float(node.find("currentTime").text) == pytest.approx(s.time(), rel=1e-12)
        com = [float(node.find(f"currentCenterOfMass/{k}").text) for k in "xyz"]
        np.testing.assert_allclose(com, s.com(), rtol=0, atol=1e-6 * robot.vox_size)
        fit = float(node.find("fitness_score").text)
        assert fit == pytest.approx(s.com()[0] - c0[0], abs=1e-6 * robot.vox_size)
        assert int(node.find("num_voxel").text) == s.counts()[0]
    best = rep.find("bestfit/filename").text
    fits = {n.tag: float(n.find("fitness_score").text) for n in rep.find("detail")}
    assert best.split(".")[0] == max(fits, key=fits.get)


def test_runner_history_text(tmp_path):
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    robot = wl.solid_block(3, stop_time=0.005, record_step=10)
    (tmp_path / "base.vxa").write_text(wl.to_vxa(robot))
    (tmp_path / "r.vxd").write_text("<VXD>\n</VXD>\n")
    r = subprocess.run([exe, "-i", str(tmp_path), "-o", str(tmp_path / "o.xml")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("<<<Step")]
    assert lines and lines[0].startswith("<<<Step0 Time:")
    # every surface voxel (26 of 27) is one ';'-terminated record of 15 comma fields
    body = lines[0].split(">>>", 1)[1].rsplit("<<<>>>", 1)[0]
    recs = [x for x in body.split(";") if x]
    assert len(recs) == 26
    assert all(len(x.rstrip(",").split(",")) == 15 for x in recs)


def test_runner_force_field_matches_oracle(tmp_path):
    """Simulator/ForceField in the VXA: the runner's token programs (built from the
    XML the way ParseMathTree lays them out) move the robot as the oracle does."""
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    C = lambda v: ("mtCONST", v)  # noqa: E731
    V = lambda n: ("mtVAR", n)  # noqa: E731
    ff = [("mtMUL", C(1e-2), ("mtCOS", ("mtMUL", C(20.0), V("t")))),
          ("mtMUL", C(-0.3), ("mtSUB", V("y"), C(0.02))),
          ("mtDIV", ("mtSQRT", V("num_voxel")), C(2e3))]
    rng = np.random.default_rng(8)
    mats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=3e5, nu=0.35, cte=0.0)]
    robot = wl.bernoulli_body(rng, (4, 4, 3), 0.85, mats, random_phase=True, temp_vary=True, temp_amplitude=20.0,
                              stop_time=0.01, fitness_x=True, force_field=ff)
    (tmp_path / "base.vxa").write_text(wl.to_vxa(robot))
    (tmp_path / "r.vxd").write_text("<VXD>\n</VXD>\n")
    out = tmp_path / "report.xml"
    r = subprocess.run([exe, "-i", str(tmp_path), "-o", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    node = ET.parse(out).getroot().find("detail/r")
    s, c0, _ = _oracle_until(robot, 0.01)
    com = [float(node.find(f"currentCenterOfMass/{k}").text) for k in "xyz"]
    np.testing.assert_allclose(com, s.com(), rtol=0, atol=1e-6 * robot.vox_size)
    free = wl.Robot(**{**robot.__dict__, "force_field": None})
    f, _, _ = _oracle_until(free, 0.01)
    assert np.abs(f.com() - s.com()).max() > 1e-4 * robot.vox_size  # the field moved the robot


def test_runner_cilia_matches_oracle(tmp_path):
    """EnableCilia with Structure/BaseCiliaForce and ShiftCiliaForce rows and per-material
    Cilia / TurnOnCiliaAfterThisManySeconds, through the runner, against the oracle."""
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    rng = np.random.default_rng(12)
    mats = [wl.Material(E=1e6, nu=0.35, cte=0.01, cilia=1.0),
            wl.Material(E=3e5, nu=0.35, cilia=0.7, cilia_on_after=0.004)]
    robot = wl.bernoulli_body(rng, (4, 4, 3), 0.85, mats, random_phase=True, temp_vary=True, temp_amplitude=20.0,
                              stop_time=0.01, fitness_x=True)
    robot.enable_cilia = True
    robot.cilia_base = 2e-2 * rng.standard_normal(robot.grid.shape + (3,))
    robot.cilia_shift = 1e-2 * rng.standard_normal(robot.grid.shape + (3,))
    (tmp_path / "base.vxa").write_text(wl.to_vxa(robot))
    (tmp_path / "r.vxd").write_text("<VXD>\n</VXD>\n")
    out = tmp_path / "report.xml"
    r = subprocess.run([exe, "-i", str(tmp_path), "-o", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    node = ET.parse(out).getroot().find("detail/r")
    s, _, _ = _oracle_until(robot, 0.01)
    com = [float(node.find(f"currentCenterOfMass/{k}").text) for k in "xyz"]
    np.testing.assert_allclose(com, s.com(), rtol=0, atol=1e-6 * robot.vox_size)
    free = wl.Robot(**{**robot.__dict__, "enable_cilia": False})
    f, _, _ = _oracle_until(free, 0.01)
    assert np.abs(f.com() - s.com()).max() > 1e-4 * robot.vox_size  # the cilia moved the robot
