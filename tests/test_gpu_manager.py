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


def test_runner_material_models_match_oracle(tmp_path):
    """MatModel 2 (bilinear, Plastic_Mod / Yield_Stress / Fail_Stress) and MatModel 3
    (SSData points) read from the VXA by the runner: the report matches the oracle
    running the same robot, and the plastic materials move it differently from linear
    ones of the same initial modulus."""
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    rng = np.random.default_rng(12)
    bil = wl.Material(E=1e5, nu=0.35, cte=0.01, model=2, plastic_mod=2e4, yield_stress=120.0, fail_stress=-1.0)
    dat = wl.Material(E=0, nu=0.35, cte=0.01, model=3, ss_strain=(0, 0.002, 0.006, 0.02),
                      ss_stress=(0, 200.0, 450.0, 600.0))
    robot = wl.bernoulli_body(rng, (5, 4, 3), 0.85, [bil, dat, wl.Material(E=1e5, nu=0.35)], random_phase=True,
                              temp_vary=True, temp_amplitude=10.0, temp_period=0.02, enable_expansion=1,
                              stop_time=0.01, fitness_x=True)
    (tmp_path / "base.vxa").write_text(wl.to_vxa(robot))
    (tmp_path / "r.vxd").write_text("<VXD>\n</VXD>\n")
    out = tmp_path / "report.xml"
    r = subprocess.run([exe, "-i", str(tmp_path), "-o", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    node = ET.parse(out).getroot().find("detail/r")
    s, c0, _ = _oracle_until(robot, 0.01)
    assert float(node.find("currentTime").text) == pytest.approx(s.time(), rel=1e-12)
    com = [float(node.find(f"currentCenterOfMass/{k}").text) for k in "xyz"]
    np.testing.assert_allclose(com, s.com(), rtol=0, atol=1e-6 * robot.vox_size)
    assert np.count_nonzero(s.link_offsets()) > 0  # some links yielded
    lin = wl.Robot(**{**robot.__dict__, "materials": [wl.Material(E=1e5, nu=0.35, cte=0.01),
                                                      wl.Material(E=1e5, nu=0.35, cte=0.01),
                                                      wl.Material(E=1e5, nu=0.35)]})
    f, _, _ = _oracle_until(lin, 0.01)
    assert np.abs(f.com() - s.com()).max() > 1e-4 * robot.vox_size


def test_runner_boundary_conditions_match_oracle(tmp_path):
    """<Environment><Boundary_Conditions> read by the runner: a clamped, loaded
    cantilever and an actuated body with partial DOF fixes, against the oracle."""
    import golden_cases
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    for name in ("beam10_clamped_bcs", "bern6_partial_bcs"):
        robot, _ = golden_cases.load(name)
        robot.stop_time = 0.01
        d = tmp_path / name
        d.mkdir()
        (d / "base.vxa").write_text(wl.to_vxa(robot))
        (d / "r.vxd").write_text("<VXD>\n</VXD>\n")
        out = d / "report.xml"
        r = subprocess.run([exe, "-i", str(d), "-o", str(out)], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        node = ET.parse(out).getroot().find("detail/r")
        s, _, _ = _oracle_until(robot, 0.01)
        com = [float(node.find(f"currentCenterOfMass/{k}").text) for k in "xyz"]
        np.testing.assert_allclose(com, s.com(), rtol=0, atol=1e-6 * robot.vox_size)
        free = wl.Robot(**{**robot.__dict__, "bcs": None})
        f, _, _ = _oracle_until(free, 0.01)
        assert np.abs(f.com() - s.com()).max() > 1e-4 * robot.vox_size, name  # the regions acted


def test_runner_signals_match_oracle(tmp_path):
    """Simulator/EnableSignals with pacemaker materials and ShiftCiliaForce rows read by
    the runner from the VXA: the report matches the oracle running the same robot, and
    the signals moved it."""
    import golden_cases
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    robot, _ = golden_cases.load("bern6_signals_cilia")
    robot.stop_time = 0.008
    (tmp_path / "base.vxa").write_text(wl.to_vxa(robot))
    (tmp_path / "r.vxd").write_text("<VXD>\n</VXD>\n")
    out = tmp_path / "report.xml"
    r = subprocess.run([exe, "-i", str(tmp_path), "-o", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    node = ET.parse(out).getroot().find("detail/r")
    s, _, _ = _oracle_until(robot, 0.008)
    com = [float(node.find(f"currentCenterOfMass/{k}").text) for k in "xyz"]
    np.testing.assert_allclose(com, s.com(), rtol=0, atol=1e-6 * robot.vox_size)
    quiet, _, _ = _oracle_until(wl.Robot(**{**robot.__dict__, "enable_signals": False}), 0.008)
    assert np.abs(quiet.com() - s.com()).max() > 1e-4 * robot.vox_size


def test_runner_attachment_matches_oracle(tmp_path):
    """Simulator/AttachDetach/EnableAttach with SafetyGuard, an AttachCondition program and
    Sticky materials read by the runner from the VXA: the pieces dropped on the plate link
    up and the report matches the oracle running the same robot; without attachment the
    robot ends elsewhere."""
    import golden_cases
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    robot, _ = golden_cases.load("sticky_drop_attach")
    robot.stop_time = 0.06
    (tmp_path / "base.vxa").write_text(wl.to_vxa(robot))
    (tmp_path / "r.vxd").write_text("<VXD>\n</VXD>\n")
    out = tmp_path / "report.xml"
    r = subprocess.run([exe, "-i", str(tmp_path), "-o", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    node = ET.parse(out).getroot().find("detail/r")
    s, _, _ = _oracle_until(robot, 0.06)
    assert s.counts()[1] > ob.oracle_sim(robot).counts()[1]  # links were made
    com = [float(node.find(f"currentCenterOfMass/{k}").text) for k in "xyz"]
    np.testing.assert_allclose(com, s.com(), rtol=0, atol=1e-6 * robot.vox_size)
    loose, _, _ = _oracle_until(wl.Robot(**{**robot.__dict__, "enable_attach": False}), 0.06)
    assert np.abs(loose.com() - s.com()).max() > 1e-4 * robot.vox_size


def test_runner_sub_batches_run_concurrently(tmp_path):
    """VX3_SimulationManager::start runs every sub-batch at once, one host thread and
    context per device: four robots dealt round-robin into two sub-batches, both on
    device 0 (one GPU here), give exactly the results of the single sub-batch run --
    robots are independent, and a robot's result does not depend on its batch."""
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    rng = np.random.default_rng(31)
    mats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=3e5, nu=0.35, cte=0.0)]
    robots = [wl.bernoulli_body(rng, tuple(int(x) for x in rng.integers(4, 7, size=3)), 0.8, mats, random_phase=True,
                                temp_vary=True, temp_amplitude=39.0, stop_time=0.02, fitness_x=True,
                                enable_collision=bool(i % 2)) for i in range(4)]
    (tmp_path / "base.vxa").write_text(wl.to_vxa(robots[0]))
    for i, r in enumerate(robots):
        (tmp_path / f"r{i}.vxd").write_text(wl.to_vxd(r))
    reports = {}
    for tag, extra in (("one", ["--devices", "1"]), ("two", ["--devices", "2", "--device-map", "0,0"])):
        out = tmp_path / f"{tag}.xml"
        p = subprocess.run([exe, "-i", str(tmp_path), "-o", str(out)] + extra, capture_output=True, text=True,
                           timeout=600)
        assert p.returncode == 0, p.stderr
        reports[tag] = {n.tag: {c.tag: c.text for c in n if len(c) == 0} for n in ET.parse(out).getroot().find("detail")}
    assert sorted(reports["one"]) == [f"r{i}" for i in range(4)]
    assert reports["one"] == reports["two"]


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


def _eval_tree(tree, v):
    """A math tree over the operators these tests use, operands in document order."""
    op = tree[0]
    if op == "mtCONST":
        return float(tree[1])
    if op == "mtVAR":
        return float(v.get(tree[1], 0.0))
    a = [_eval_tree(c, v) for c in tree[1:]]
    return {"mtADD": lambda: a[0] + a[1], "mtSUB": lambda: a[0] - a[1], "mtMUL": lambda: a[0] * a[1],
            "mtDIV": lambda: a[0] / a[1], "mtGREATERTHAN": lambda: float(a[0] > a[1]),
            "mtLESSTHAN": lambda: float(a[0] < a[1])}[op]()


def _reference_run(robot, stop, max_steps=100000, fresh_com=False):
    """CUDA_Simulation (VX3_SimulationManager.cu:54-118) over the oracle: StopConditionMet
    before every step reads currentCenterOfMass, which doTimeStep refreshes only when the
    step count is a multiple of CycleStep = int(TempPeriod / dt) (VX3_VoxelyzeKernel.cu:
    313-320); a SecondaryExperiment takes the initial COM (that value) and the initial
    voxel positions again at the end of the first step that starts after
    ReinitializeInitialPositionAfterThisManySeconds (:344-348).  fresh_com=True reads the
    current COM instead (what the runner must NOT do)."""
    s = ob.oracle_sim(robot)
    nv = s.counts()[0]
    com0 = s.com()
    com_s, init, n, reset = com0.copy(), s.voxels()["pos"].copy(), 0, False
    while n < max_steps:
        t = s.time()
        c = s.com() if fresh_com else com_s
        if _eval_tree(stop, dict(x=c[0], y=c[1], z=c[2], t=t, num_voxel=nv)) > 0:
            break
        s.step(1)
        n += 1
        cyc = int(robot.temp_period / float(np.float32(s.dt())))
        if cyc > 0 and n % cyc == 0:
            com_s = s.com()
        if robot.secondary_experiment and not reset and robot.reinit_after < t:
            reset = True
            com0, init = com_s.copy(), s.voxels()["pos"].copy()
    return s, n, com0, init


def _run_runner(tmp_path, robot):
    vbuild.build()
    exe = os.path.join(os.path.dirname(vbuild.LIB), "vx3g_sim")
    (tmp_path / "base.vxa").write_text(wl.to_vxa(robot))
    (tmp_path / "r.vxd").write_text("<VXD>\n</VXD>\n")
    out = tmp_path / "report.xml"
    r = subprocess.run([exe, "-i", str(tmp_path), "-o", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return ET.parse(out).getroot().find("detail/r")


def _xyz(node, tag):
    return np.array([float(node.find(f"{tag}/{k}").text) for k in "xyz"])


def test_runner_com_stop_condition_reads_the_sampled_com(tmp_path):
    """A StopConditionFormula on the centre of mass stops where the reference's does: the
    COM it reads is the one sampled every int(TempPeriod/dt) steps, not the current one."""
    rng = np.random.default_rng(14)
    mats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=3e5, nu=0.35)]
    robot = wl.bernoulli_body(rng, (4, 3, 3), 0.9, mats, random_phase=True, temp_vary=True, temp_amplitude=20.0,
                              temp_period=0.003, z_offset=2, fitness_x=True)
    z0 = ob.oracle_sim(robot).com()[2]
    robot.stop_formula = ("mtLESSTHAN", ("mtVAR", "z"), ("mtCONST", z0 - 0.004))
    s, n, c0, _ = _reference_run(robot, robot.stop_formula)
    _, n_fresh, _, _ = _reference_run(robot, robot.stop_formula, fresh_com=True)
    assert n_fresh < n  # the sampled COM lags: the two readings stop at different steps
    node = _run_runner(tmp_path, robot)
    assert float(node.find("currentTime").text) == pytest.approx(s.time(), rel=1e-12)
    np.testing.assert_allclose(_xyz(node, "currentCenterOfMass"), s.com(), rtol=0, atol=1e-6 * robot.vox_size)
    np.testing.assert_allclose(_xyz(node, "initialCenterOfMass"), c0, rtol=0, atol=1e-9 * robot.vox_size)


def test_runner_secondary_experiment_matches_oracle(tmp_path):
    """SecondaryExperiment through the runner: a material leaves the simulation
    (RemoveFromSimulationAfterThisManySeconds) and the initial COM and positions are taken
    again (ReinitializeInitialPositionAfterThisManySeconds), as the reference's loop does."""
    rng = np.random.default_rng(15)
    mats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=3e5, nu=0.35, remove_after=0.002),
            wl.Material(E=5e5, nu=0.35, is_measured=0)]
    robot = wl.bernoulli_body(rng, (5, 4, 3), 0.9, mats, random_phase=True, temp_vary=True, temp_amplitude=20.0,
                              temp_period=0.001, enable_collision=True, stop_time=0.006, fitness_x=True, z_offset=1)
    robot.secondary_experiment = True
    robot.reinit_after = 0.003
    robot.stop_formula = ("mtSUB", ("mtVAR", "t"), ("mtCONST", 0.006))
    s, n, c0, init = _reference_run(robot, robot.stop_formula)
    node = _run_runner(tmp_path, robot)
    assert float(node.find("currentTime").text) == pytest.approx(s.time(), rel=1e-12)
    com = _xyz(node, "currentCenterOfMass")
    np.testing.assert_allclose(com, s.com(), rtol=0, atol=1e-6 * robot.vox_size)
    np.testing.assert_allclose(_xyz(node, "initialCenterOfMass"), c0, rtol=0, atol=1e-6 * robot.vox_size)
    assert float(node.find("fitness_score").text) == pytest.approx(s.com()[0] - c0[0], abs=1e-6 * robot.vox_size)
    # total_distance_of_all_voxels: measured voxels' distance from the positions at the reset
    pos = s.voxels()["pos"]
    mat = s.topology()["mat"]
    meas = np.array([robot.materials[k].is_measured for k in mat], bool)
    want = np.linalg.norm(pos[meas] - init[meas], axis=1).sum()
    assert float(node.find("total_distance_of_all_voxels").text) == pytest.approx(
        want, rel=0, abs=1e-6 * robot.vox_size * meas.sum())
    assert int(node.find("num_measured_voxel").text) == int(meas.sum())
