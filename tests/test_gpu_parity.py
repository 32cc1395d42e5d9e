"""GB300 parity: the CUDA step (through the C ABI) against the reference's
golden vectors and the CPU oracle.

Tolerances (written here, per the parity bar):
  * FP64 path, integer/index outputs (topology, ordering, surface list,
    small-angle flags, static-friction flags, divergence): exact.
  * FP64 path, positions: |dx| <= 1e-6 * voxel size per step over the compared
    horizon (the reference bar); in practice the FP64 kernels track the
    reference to ~1e-15 m, the residual being CUDA's sin/acos vs the host libm.
  * Mixed path: relative centre-of-mass error vs the FP64 path <= 1e-5.
"""

import numpy as np
import pytest

import golden_cases
import oracle_bridge as ob
from vx3g import abi
from vx3g import workloads as wl

pytestmark = pytest.mark.gpu

POS_TOL = 1e-6  # in voxel sizes


def _robot_slice(b, i, a):
    return a[b.voxel_offset[i]:b.voxel_offset[i + 1]]


@pytest.mark.parametrize("name", golden_cases.names())
def test_fp64_against_reference_golden(name):
    robot, d = golden_cases.load(name)
    b = abi.Batch([robot], abi.PRECISION_FP64)
    t = b.topology()
    n = int(b.links_in_use()[0])  # the link range holds a reserve for runtime links after these
    for k in ("ijk", "mat"):
        assert np.array_equal(t[k], d["topo_" + k]), k
    for k in ("negpos", "axis"):
        assert np.array_equal(t[k][:n], d["topo_" + k]), k
    done = 0
    for snap in d["snap_steps"]:
        snap = int(snap)
        b.step(snap - done)
        done = snap
        st, aux, lk = b.state(), b.voxel_aux(), b.links()
        n = int(b.links_in_use()[0])
        lk = {k: v[:n] for k, v in lk.items()}
        if f"s{snap}_negpos" in d.files:  # attachment: the same runtime links, in order, on the same faces
            t = b.topology()
            assert np.array_equal(t["negpos"][:n], d[f"s{snap}_negpos"])
            assert np.array_equal(t["axis"][:n], d[f"s{snap}_axis"])
        dpos = np.max(np.abs(st["pos"] - d[f"s{snap}_pos"]))
        assert dpos <= POS_TOL * robot.vox_size, f"{name}@{snap}: pos error {dpos:.3e}"
        dq = np.max(np.abs(st["orient"] - d[f"s{snap}_orient"]))
        assert dq < 1e-9, f"{name}@{snap}: orientation error {dq:.3e} (links in use {n})"
        assert np.array_equal(b.surface(), d[f"s{snap}_surface"])
        assert np.array_equal(lk["small"] & 1, d[f"s{snap}_small"])
        assert np.array_equal(aux["flags"] & 8, d[f"s{snap}_flags"] & 8)  # static friction
        np.testing.assert_allclose(aux["tempe"], d[f"s{snap}_tempe"], rtol=0, atol=1e-4)
        np.testing.assert_allclose(aux["contact"], d[f"s{snap}_contact"], rtol=1e-6, atol=1e-9)
        np.testing.assert_allclose(lk["strain"], d[f"s{snap}_strain"], rtol=0, atol=1e-6)
        np.testing.assert_allclose(b.time()[0], d[f"s{snap}_time"][0], rtol=1e-12)
        np.testing.assert_allclose(b.com()[0], d[f"s{snap}_com"], rtol=1e-12)  # measured voxels only
        assert np.float32(b.dt()[0]) == d[f"s{snap}_dt"][0]
        if f"s{snap}_signal" in d.files:  # EnableSignals: localSignal per voxel
            np.testing.assert_allclose(b.signals(), d[f"s{snap}_signal"], rtol=1e-12, atol=0)
    assert np.all(b.status() == 0)


def _seeded_batch(seed, n=3):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = tuple(int(x) for x in rng.integers(3, 7, size=3))
        mats = [wl.Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, cte=0.01) for _ in range(3)]
        out.append(wl.bernoulli_body(rng, dims, 0.7, mats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                                     enable_collision=bool(i % 2), z_offset=1))
    return out


def test_fp64_batch_matches_oracle_per_step():
    robots = _seeded_batch(11)
    b = abi.Batch(robots, abi.PRECISION_FP64)
    sims = [ob.oracle_sim(r) for r in robots]
    for step in range(1, 101):
        b.step(1)
        st = b.state()
        for i, (r, s) in enumerate(zip(robots, sims)):
            s.step(1)
            ref = s.voxels()
            err = np.max(np.abs(_robot_slice(b, i, st["pos"]) - ref["pos"]))
            assert err <= POS_TOL * r.vox_size, f"robot {i} step {step}: {err:.3e}"
    for i, s in enumerate(sims):
        np.testing.assert_allclose(b.com()[i], s.com(), rtol=1e-12)


def test_batch_with_linkless_robot_matches_oracle():
    """A robot of one voxel (no links) between two others in one batch, FP64 and mixed:
    the batch's link offsets skip it, its time step comes from its own stiffness, and every
    robot follows the oracle (FP64 within the position bar; mixed COM within 1e-5)."""
    rng = np.random.default_rng(41)
    mats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=3e5, nu=0.35, cte=0.01)]
    one = wl.Robot(grid=np.ones((1, 1, 1), np.uint8), materials=[wl.Material(E=5e5, nu=0.35, cte=0.01)],
                   phase=np.full((1, 1, 1), 0.7), temp_vary=True, temp_amplitude=39.0, enable_expansion=1,
                   z_offset=1)
    robots = [wl.bernoulli_body(rng, (4, 3, 3), 0.8, mats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                                enable_collision=True, z_offset=1),
              one, wl.solid_block(3)]
    b = abi.Batch(robots, abi.PRECISION_FP64)
    assert b.link_offset[1] == b.link_offset[2]  # no links of its own
    sims = [ob.oracle_sim(r) for r in robots]
    for _ in range(4):
        b.step(50)
        st = b.state()
        for i, (r, s) in enumerate(zip(robots, sims)):
            s.step(50)
            err = np.max(np.abs(_robot_slice(b, i, st["pos"]) - s.voxels()["pos"]))
            assert err <= POS_TOL * r.vox_size, f"robot {i}: {err:.3e}"
            assert np.float32(b.dt()[i]) == np.float32(s.dt())
    m = abi.Batch(robots, abi.PRECISION_MIXED)
    m.step(200)
    assert np.all(b.status() == 0) and np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - b.com(), axis=1) / np.linalg.norm(b.com(), axis=1)
    assert np.all(rel <= 1e-5), rel


def test_batch_invariance_and_determinism():
    robots = _seeded_batch(5, n=4)
    together = abi.Batch(robots, abi.PRECISION_FP64)
    together.step(150)
    p_all = together.state()["pos"]
    again = abi.Batch(robots, abi.PRECISION_FP64)
    again.step(150)
    assert np.array_equal(again.state()["pos"], p_all)  # bit-identical rerun
    for i, r in enumerate(robots):
        alone = abi.Batch([r], abi.PRECISION_FP64)
        alone.step(150)
        assert np.array_equal(alone.state()["pos"], _robot_slice(together, i, p_all))


def test_graph_chunks_match_single_steps():
    robots = _seeded_batch(3, n=2)
    a = abi.Batch(robots, abi.PRECISION_FP64, graph_chunk=10)
    a.step(37)
    b = abi.Batch(robots, abi.PRECISION_FP64, graph_chunk=1000)
    for _ in range(37):
        b.step(1)
    assert np.array_equal(a.state()["pos"], b.state()["pos"])
    assert np.array_equal(a.time(), b.time())


def _expanding(rng, grid_shape, p=1.0):
    """A self-colliding body: 39 C actuation with CTE 0.01 and EnableExpansion grows
    voxels to 1.39 voxel sizes, so diagonal neighbours (1.41 apart) touch."""
    mats = [wl.Material(E=2e5, nu=0.35, cte=0.01), wl.Material(E=1e6, nu=0.35, cte=0.01)]
    mask = wl.largest_component(rng.random(grid_shape) < p)
    grid = np.where(mask, rng.integers(1, 3, size=grid_shape), 0).astype(np.uint8)
    return wl.Robot(grid=grid, materials=mats, phase=rng.random(grid_shape), temp_vary=True, temp_amplitude=39.0,
                    enable_collision=True, enable_expansion=1, z_offset=1)


def test_both_list_builds_match_oracle():
    """Contact forces and positions against the oracle for a batch that uses both
    candidate-list builds: a 1030-long two-voxel strip (lattice coordinates past
    1023, so its lists come from the global hashed grid) and a small body (lists
    built per robot in shared memory)."""
    rng = np.random.default_rng(31)
    robots = [_expanding(rng, (1, 2, 1030)), _expanding(rng, (4, 5, 6), 0.85)]
    b = abi.Batch(robots, abi.PRECISION_FP64)
    sims = [ob.oracle_sim(r) for r in robots]
    for _ in range(3):
        b.step(20)
        st, aux = b.state(), b.voxel_aux()
        for i, (r, s) in enumerate(zip(robots, sims)):
            s.step(20)
            err = np.max(np.abs(_robot_slice(b, i, st["pos"]) - s.voxels()["pos"]))
            assert err <= POS_TOL * r.vox_size, f"robot {i}: {err:.3e}"
            c, ref = _robot_slice(b, i, aux["contact"]), s.last_contact()
            assert np.count_nonzero(np.abs(ref).sum(1)) > 0, f"robot {i}: no contacts"
            np.testing.assert_allclose(c, ref, rtol=1e-6, atol=1e-9 * np.abs(ref).max())
    assert np.all(b.status() == 0)
    m = abi.Batch(robots, abi.PRECISION_MIXED)
    m.step(60)
    assert np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - b.com(), axis=1) / np.linalg.norm(b.com(), axis=1)
    assert np.all(rel <= 1e-5), rel
    # the mixed step's contact forces (FP32, read back through the same getter) follow the FP64 ones
    cf, cm = b.voxel_aux()["contact"], m.voxel_aux()["contact"]
    assert np.count_nonzero(np.abs(cm).sum(1)) > 0
    np.testing.assert_allclose(cm, cf, rtol=0, atol=1e-2 * np.abs(cf).max())


def _ff(*trees):
    return list(trees)


def test_force_field_programs_are_checked():
    """Programs are validated at create: target-tracking variables are unsupported,
    an operator without operands or a program without mtEND's single value is invalid."""
    base = wl.solid_block(3)
    C = lambda v: ("mtCONST", v)  # noqa: E731
    ok = wl.Robot(**{**base.__dict__, "force_field": _ff(("mtMUL", C(1e-3), ("mtVAR", "t")), None, None)})
    abi.Batch([ok], abi.PRECISION_FP64).close()
    angle = wl.Robot(**{**base.__dict__, "force_field": _ff(("mtVAR", "angle"), None, None)})
    with pytest.raises(abi.Vx3gError, match="target tracking"):
        abi.Batch([angle], abi.PRECISION_FP64)
    lib = abi.load()
    d, keep = abi.robot_desc(base)
    for toks in ([(5, 0, 0.0), (0, 0, 0.0)],                 # mtADD with nothing to add
                 [(1, 0, 1.0), (1, 0, 2.0), (0, 0, 0.0)],    # two values left at mtEND
                 [(1, 0, 1.0)] * 300):                        # no mtEND
        arr = np.array(toks, dtype=[("op", np.int32), ("reserved", np.int32), ("value", np.float64)])
        d.force_field[2] = arr.ctypes.data
        bd = abi.BatchDesc(1, abi.ctypes.pointer(d), abi.PRECISION_FP64, 0, 100)
        st = abi.ctypes.c_int(0)
        assert not lib.vx3g_create(abi.ctypes.byref(bd), abi.ctypes.byref(st))
        assert st.value == -1, lib.vx3g_last_error()


def test_adjoint_with_force_fields():
    """record() refuses a force field that reads the position; a time-only field is
    part of the recomputed forward step, so backward() still matches central
    differences (4 phases, 120 steps, eps = 1e-6, within 3%)."""
    base = wl.c4_differentiable(0)[0]
    C = lambda v: ("mtCONST", v)  # noqa: E731
    pos = wl.Robot(**{**base.__dict__, "force_field": _ff(None, ("mtMUL", C(-0.1), ("mtVAR", "y")), None)})
    b = abi.Batch([pos], abi.PRECISION_FP64)
    with pytest.raises(abi.Vx3gError, match="position"):
        b.record(10, 5)
    ff = _ff(("mtMUL", C(3e-3), ("mtSIN", ("mtMUL", C(31.4), ("mtVAR", "t")))), None,
             ("mtMUL", C(1e-8), ("mtVAR", "num_voxel")))
    robot = wl.Robot(**{**base.__dict__, "force_field": ff})
    n = 120
    b = abi.Batch([robot], abi.PRECISION_FP64)
    b.record(n, 40)
    gp, _ = b.backward(np.array([[-1.0, 0.0, 0.0]]))
    ph = robot.phase.reshape(-1)
    idx = np.flatnonzero(robot.grid.reshape(-1) > 0)
    rng = np.random.default_rng(3)
    errs = []
    for k in rng.choice(len(idx), 4, replace=False):
        cell, eps = idx[k], 1e-6
        f = []
        for sgn in (1, -1):
            p = ph.copy()
            p[cell] += sgn * eps
            r2 = wl.Robot(**{**robot.__dict__, "phase": p.reshape(robot.phase.shape)})
            c = abi.Batch([r2], abi.PRECISION_FP64)
            c0 = c.com()[0, 0]
            c.step(n)
            f.append(-(c.com()[0, 0] - c0))
        fd = (f[0] - f[1]) / (2 * eps)
        errs.append(abs(gp[k] - fd) / max(abs(fd), abs(gp[k]), 1e-2 * np.abs(gp).max()))
    assert np.median(errs) <= 0.03, errs


def test_cilia_mixed_and_adjoint_guard():
    """Cilia in a mixed-precision context stay within the mixed COM bar of the FP64
    run, and the adjoint refuses cilia (its derivative is not formed)."""
    robot, _ = golden_cases.load("bern5_cilia")
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    f.step(300)
    m.step(300)
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-5), rel
    with pytest.raises(abi.Vx3gError, match="cilia"):
        abi.Batch([robot], abi.PRECISION_FP64).record(10, 5)


def test_detach_surface_and_guards():
    """EnableDetach: the surface grows as links detach (mixed and FP64 agree on it),
    the adjoint refuses a changing link table."""
    robot, d = golden_cases.load("block4_detach")
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    n0 = len(f.surface())
    f.step(300)
    m.step(300)
    assert len(f.surface()) > n0
    assert np.array_equal(f.surface(), d["s300_surface"])
    assert np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-4), rel
    with pytest.raises(abi.Vx3gError, match="detach"):
        abi.Batch([robot], abi.PRECISION_FP64).record(10, 5)


@pytest.mark.parametrize("name", ["bern6_removal", "block4_detach_cilia"])
def test_changing_surface_mixed_matches_fp64(name):
    """Material removal (SecondaryExperiment) and detach with cilia: the mixed-precision
    kernels follow the FP64 ones (same surface, COM within 1e-5 relative), removed voxels
    stop moving, and the adjoint refuses a changing link table."""
    robot, d = golden_cases.load(name)
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    f.step(200)
    m.step(200)
    p200 = f.state()["pos"]
    f.step(100)
    m.step(100)
    assert np.all(f.status() == 0) and np.all(m.status() == 0)
    assert np.array_equal(f.surface(), d["s300_surface"])
    assert np.array_equal(m.surface(), d["s300_surface"])
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-5), rel
    if robot.secondary_experiment:
        t = f.topology()
        gone = np.array([robot.materials[k].remove_after > 0 and robot.materials[k].remove_after < 0.0052
                         for k in t["mat"]])
        assert gone.any()
        assert np.array_equal(f.state()["pos"][gone], p200[gone])  # removed by step 200: frozen since
        assert not np.isin(np.nonzero(gone)[0], f.surface()).any()
        gone300 = np.array([0 < robot.materials[k].remove_after < 0.0077 for k in t["mat"]])
        lk = f.links()
        ends = t["negpos"]
        assert np.all(((lk["small"] & 2) != 0) == (gone300[ends[:, 0]] | gone300[ends[:, 1]]))
    with pytest.raises(abi.Vx3gError, match="not implemented"):
        abi.Batch([robot], abi.PRECISION_FP64).record(10, 5)


@pytest.mark.parametrize("name", ["bilinear_cantilever_plastic", "bern5_data_bilinear", "bern4_data_bilinear_poisson"])
def test_nonlinear_materials_mixed_matches_fp64(name):
    """Bilinear and data-point stress-strain models with plastic unloading: the
    mixed-precision kernels follow the FP64 ones (COM within 1e-5 relative, small-angle
    states identical at the end of the golden horizon), and the adjoint refuses them."""
    robot, d = golden_cases.load(name)
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    n = int(d["snap_steps"][-1])
    f.step(n)
    m.step(n)
    assert np.all(f.status() == 0) and np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-5), rel
    lf, lm = f.links(), m.links()
    plastic = lf["maxstrain"] > 0
    assert plastic.any()
    np.testing.assert_allclose(lm["maxstrain"], lf["maxstrain"], rtol=0, atol=1e-5)
    with pytest.raises(abi.Vx3gError, match="not implemented"):
        abi.Batch([robot], abi.PRECISION_FP64).record(10, 5)


def test_thermal_delay_mixed_matches_fp64():
    """TurnOnThermalExpansionAfterThisManySeconds: the delayed materials keep their initial
    temperature until their turn-on time in both precisions, switch on in the same step,
    and the mixed step's temperatures (the actuation phase carried as FP32 cycles) stay
    within 1e-4 degrees of the FP64 step's; COM within 1e-5 relative."""
    robot, d = golden_cases.load("bern5_thermal_delay")
    g, _ = robot.padded()
    cells = g.reshape(-1)
    mat = cells[cells > 0] - 1
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    for snap in (100, 200, 300):
        f.step(100)
        m.step(100)
        tf, tm = f.voxel_aux()["tempe"], m.voxel_aux()["tempe"]
        np.testing.assert_allclose(tf, d[f"s{snap}_tempe"], rtol=0, atol=1e-4)
        for k, m_on in enumerate(robot.materials):
            sel = mat == k
            on = m_on.thermal_on_after <= float(d[f"s{snap}_time"][0])
            assert np.any(tf[sel] != 0) == on, (snap, k)
            assert np.array_equal(tm[sel] != 0, tf[sel] != 0), (snap, k)
        np.testing.assert_allclose(tm, tf, rtol=0, atol=1e-4)
    assert np.all(f.status() == 0) and np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-5), rel


def test_static_expansion_mixed_matches_fp64():
    """Thermal/TempEnabled without VaryTempEnabled: every voxel starts, and stays, at
    TempAmplitude above TempBase (a bimetal block, one material expanded by 20%, bends as it
    drops); the mixed step follows the FP64 one (COM within 1e-5 relative)."""
    robot, d = golden_cases.load("bimetal_static_expansion")
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    f.step(300)
    m.step(300)
    assert np.all(f.voxel_aux()["tempe"] == np.float32(robot.temp_amplitude))
    assert np.all(m.voxel_aux()["tempe"] == np.float32(robot.temp_amplitude))
    assert np.all(f.status() == 0) and np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-5), rel


@pytest.mark.parametrize("name", ["bern6_damping_settings", "bern6_density_measured_fixed"])
def test_settings_mixed_matches_fp64(name):
    """Settings every other case leaves at their defaults -- global (slow) damping, bond and
    collision damping other than 1, DtFrac 0.5 and a weaker gravity; densities, Poisson's
    ratios, a material left out of the centre of mass and Fixed voxels -- on actuated,
    self-colliding bodies: the mixed step follows the FP64 one (COM within 1e-5 relative,
    contact forces on the same voxels)."""
    robot, d = golden_cases.load(name)
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    f.step(300)
    m.step(300)
    assert np.all(f.status() == 0) and np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-5), rel
    cf, cm = f.voxel_aux()["contact"], m.voxel_aux()["contact"]
    assert np.array_equal(np.abs(cf).sum(1) > 0, np.abs(cm).sum(1) > 0)


def test_signals_mixed_matches_fp64():
    """EnableSignals with shifting cilia: the mixed-precision context carries the same
    signals (they depend on time, links and materials only) and follows the FP64 COM
    within 1e-5 relative; the adjoint refuses signals."""
    robot, d = golden_cases.load("bern6_signals_cilia")
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    f.step(400)
    m.step(400)
    assert np.array_equal(f.signals(), m.signals())
    assert np.count_nonzero(f.signals()) > 0
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-5), rel
    with pytest.raises(abi.Vx3gError, match="not implemented"):
        abi.Batch([robot], abi.PRECISION_FP64).record(10, 5)


def _com_links(robot, precision, steps, nudge=0.0, seed=1):
    b = abi.Batch([robot], precision)
    if nudge:
        st = b.state()
        st["pos"] += nudge * np.random.default_rng(seed).choice([-1.0, 1.0], size=st["pos"].shape)
        b.set_state(**st)
    b.step(steps)
    assert np.all(b.status() == 0)
    n = int(b.links_in_use()[0])
    return b.com(), b.topology()["negpos"][:n]


@pytest.mark.parametrize("name", ["sticky_drop_attach", "bimorph_u3_attach"])
def test_attach_mixed_matches_fp64(name):
    """EnableAttach in mixed precision against FP64.  The bending U shapes are not chaotic:
    the mixed kernels make the FP64 (and the reference's) runtime links and follow the FP64
    COM within 1e-5 relative.  The pieces dropped on a plate on the floor are: a 1e-9 m
    nudge of the FP64 start moves the COM by 1.5e-5 to 1.4e-4 relative (by the nudge's
    signs) through stick/slip at landing, so there the mixed error must stay within three
    times the largest spread of four nudged FP64 runs (and the links made are the FP64
    run's wherever the nudged FP64 runs make them too).  The adjoint refuses attachment."""
    robot, d = golden_cases.load(name)
    steps = int(d["snap_steps"][-1])
    c64, l64 = _com_links(robot, abi.PRECISION_FP64, steps)
    cmx, lmx = _com_links(robot, abi.PRECISION_MIXED, steps)
    assert len(l64) == len(d[f"s{steps}_negpos"]) > len(d["topo_negpos"])
    rel = float(np.linalg.norm(cmx - c64) / np.linalg.norm(c64))
    if name == "bimorph_u3_attach":
        assert np.array_equal(lmx, l64)
        assert rel <= 1e-5, rel
    else:
        floor, same = 0.0, True
        for seed in range(4):
            cnd, lnd = _com_links(robot, abi.PRECISION_FP64, steps, nudge=1e-9, seed=seed)
            floor = max(floor, float(np.linalg.norm(cnd - c64) / np.linalg.norm(c64)))
            same = same and np.array_equal(lnd, l64)
        if same:
            assert np.array_equal(lmx, l64)
        assert rel <= max(1e-5, 3 * floor), (rel, floor)
    with pytest.raises(abi.Vx3gError, match="not implemented"):
        abi.Batch([robot], abi.PRECISION_FP64).record(10, 5)


def _sticky_scene(rng, nx, pieces, attach=True):
    """A sticky plate nx long on the floor with `pieces` random sticky blocks dropped on it
    from two cells up, some of a second sticky material, some not sticky; attach conditions
    on time and height."""
    g = np.zeros((6, 4, nx), np.uint8)
    g[0, :, :] = 1
    for k in range(pieces):
        x = int(rng.integers(0, nx - 2))
        h = int(rng.integers(1, 3))
        mat = 2 if k % 5 == 4 else 3 if k % 7 == 6 else 1
        g[2:2 + h, int(rng.integers(0, 3)), x:x + int(rng.integers(1, 3))] = mat
    mats = [wl.Material(E=1e5, nu=0.0, sticky=1, mu_static=0.5, mu_kinetic=0.3),
            wl.Material(E=2e5, nu=0.0, sticky=1), wl.Material(E=1e5, nu=0.0)]
    return wl.Robot(grid=g, materials=mats, volume_effects=False, enable_collision=True, enable_attach=attach,
                    safety_guard=int(rng.integers(20, 200)),
                    attach_conditions=[("mtGREATERTHAN", ("mtVAR", "t"), ("mtCONST", 0.003)),
                                       ("mtLESSTHAN", ("mtVAR", "z"), ("mtCONST", 0.05))])


def test_attach_batch_matches_oracle():
    """Attaching robots mixed with others in one batch, on both list builds (a robot longer
    than 512 cells is rebuilt on the global hashed grid): per robot the FP64 kernels make the
    oracle's runtime links in the oracle's order and keep its trajectory."""
    rng = np.random.default_rng(31)
    robots = [_sticky_scene(rng, 14, 6), wl.solid_block(3), _sticky_scene(rng, 520, 60),
              golden_cases.load("bimorph_u3_attach")[0], _sticky_scene(rng, 20, 8, attach=False)]
    b = abi.Batch(robots, abi.PRECISION_FP64)
    steps = 500
    b.step(steps)
    st, t, use = b.state(), b.topology(), b.links_in_use()
    made = 0
    for i, r in enumerate(robots):
        o = ob.oracle_sim(r)
        n0 = o.counts()[1]
        o.step(steps)
        ot = o.topology()
        lo = b.link_offset[i]
        assert use[i] == o.counts()[1], i
        assert np.array_equal(t["negpos"][lo:lo + use[i]], ot["negpos"] + b.voxel_offset[i]), i
        assert np.array_equal(t["axis"][lo:lo + use[i]], ot["axis"]), i
        err = np.max(np.abs(_robot_slice(b, i, st["pos"]) - o.voxels()["pos"]))
        assert err <= POS_TOL * r.vox_size, (i, err)
        made += int(use[i]) - n0
    assert made >= 10, made
    assert np.all(b.status() == 0)


def test_attach_inputs_are_checked():
    """Attachment needs collisions, and a Sticky material must be linear with Poisson's
    ratio 0 (the runtime link's transverse area is the unstrained one)."""
    for bad in ("collision", "poisson", "bilinear"):
        r = golden_cases.load("sticky_drop_attach")[0]
        if bad == "collision":
            r.enable_collision = False
        elif bad == "poisson":
            r.volume_effects = True
            r.materials[0].nu = 0.3
        else:
            m = r.materials[0]
            m.model, m.plastic_mod, m.yield_stress, m.fail_stress = 2, 2e4, 50.0, -1.0
        with pytest.raises(abi.Vx3gError, match="attach|Sticky"):
            abi.Batch([r], abi.PRECISION_FP64)
    robot, d = golden_cases.load("sticky_drop_attach")
    assert abi.Batch([robot], abi.PRECISION_FP64).links_in_use()[0] == len(d["topo_negpos"])


@pytest.mark.parametrize("name", ["beam10_clamped_bcs", "bern6_partial_bcs"])
def test_boundary_conditions_mixed_matches_fp64(name):
    """Boundary-condition externals (fully clamped voxels, fixed translations with a
    displacement, all and partial rotation fixes, region forces and torques): the
    mixed-precision kernels follow the FP64 ones (COM within 1e-5 relative), the
    fully fixed voxels sit exactly at their prescribed pose in both, and the adjoint
    refuses them."""
    robot, d = golden_cases.load(name)
    f = abi.Batch([robot], abi.PRECISION_FP64)
    m = abi.Batch([robot], abi.PRECISION_MIXED)
    n = int(d["snap_steps"][-1])
    p0 = f.state()["pos"]
    f.step(n)
    m.step(n)
    assert np.all(f.status() == 0) and np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - f.com(), axis=1) / np.linalg.norm(f.com(), axis=1)
    assert np.all(rel <= 1e-5), rel
    if name == "beam10_clamped_bcs":
        clamp = f.topology()["ijk"][:, 0] == 0
        for b, tol in ((f, 0.0), (m, 1e-12)):  # mixed: a double as an FP32 hi/lo pair (~48 bits)
            st = b.state()
            assert np.max(np.abs(st["pos"][clamp] - p0[clamp])) <= tol
            assert np.max(np.abs(st["orient"][clamp] - np.array([1.0, 0, 0, 0]))) <= tol
            assert np.all(st["linmom"][clamp] == 0)
    with pytest.raises(abi.Vx3gError, match="not implemented"):
        abi.Batch([robot], abi.PRECISION_FP64).record(10, 5)


def test_mixed_com_error_vs_fp64():
    rng = np.random.default_rng(21)
    mats = [wl.Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, cte=0.01) for _ in range(4)]
    robots = [wl.bernoulli_body(rng, tuple(int(x) for x in rng.integers(4, 11, size=3)), 0.7, mats,
                                random_phase=True, temp_vary=True, temp_amplitude=39.0) for _ in range(6)]
    f = abi.Batch(robots, abi.PRECISION_FP64)
    m = abi.Batch(robots, abi.PRECISION_MIXED)
    c0 = f.com()
    f.step(2000)
    m.step(2000)
    cf, cm = f.com(), m.com()
    disp = np.linalg.norm(cf - c0, axis=1)
    rel = np.linalg.norm(cm - cf, axis=1) / np.linalg.norm(cf, axis=1)
    assert np.all(rel <= 1e-5), rel
    assert np.all(disp > 0)


def test_divergence_freezes_robot():
    # an unstable step (DtFrac far above 1) makes the link strain blow up
    bad = wl.solid_block(3, dt_frac=5.0)
    good = wl.solid_block(3)
    b = abi.Batch([bad, good], abi.PRECISION_FP64)
    s = ob.oracle_sim(bad)
    done = s.step(400)
    b.step(400)
    st = b.status()
    assert st[0] == abi.ROBOT_DIVERGED and st[1] == abi.ROBOT_OK
    assert done < 400
    assert np.isclose(b.time()[0], s.time(), rtol=1e-12)  # frozen at the same step count


def test_full_size_single_body_properties():
    """64^3 Bernoulli(0.6) body with collisions (the single-large-body workload):
    momentum balance without gravity/floor, antisymmetric contact forces, and a
    bit-identical rerun."""
    rng = np.random.default_rng(0)
    mats = [wl.Material(E=1e6, nu=0.35), wl.Material(E=1e6, nu=0.35, cte=0.01)]
    r = wl.bernoulli_body(rng, (64, 64, 64), 0.6, mats, temp_vary=True, temp_amplitude=39.0, enable_collision=True,
                          floor=False, grav_acc=0.0, slow_damping=0.0, enable_expansion=1)
    runs = []
    for _ in range(2):
        b = abi.Batch([r], abi.PRECISION_MIXED)
        b.step(200)
        runs.append(b)
    st = runs[0].state()
    assert np.array_equal(st["pos"], runs[1].state()["pos"])
    contact = runs[0].voxel_aux()["contact"]
    assert np.count_nonzero(np.abs(contact).sum(1)) > 0
    assert np.all(np.abs(contact.sum(0)) <= 1e-9 * np.abs(contact).sum())
    p = st["linmom"].sum(0)
    assert np.all(np.abs(p) <= 1e-6 * np.abs(st["linmom"]).sum())
    assert np.all(runs[0].status() == 0)


def test_settings_mix_batch_matches_oracle():
    """Eight seeded robots over densities, Poisson's ratios, isMeasured, thermal delays,
    Fixed voxels, lattice sizes, DtFrac, damping, gravity and static temperature, in one
    batch: the FP64 kernels follow the oracle robot by robot (positions within 1e-6 voxel
    sizes, centres of mass to 1e-12), and the mixed kernels follow the FP64 ones (COM within
    1e-5 relative)."""
    import feature_mix
    robots = [feature_mix.robot_settings(s) for s in range(8)]
    b = abi.Batch(robots, abi.PRECISION_FP64)
    sims = [ob.oracle_sim(r) for r in robots]
    for _ in range(4):
        b.step(60)
        pos, com = b.state()["pos"], b.com()
        for i, (r, s) in enumerate(zip(robots, sims)):
            s.step(60)
            err = np.max(np.abs(_robot_slice(b, i, pos) - s.voxels()["pos"]))
            assert err <= POS_TOL * r.vox_size, f"robot {i}: {err:.3e}"
            np.testing.assert_allclose(com[i], s.com(), rtol=1e-12, atol=1e-15)
    m = abi.Batch(robots, abi.PRECISION_MIXED)
    m.step(240)
    assert np.all(b.status() == 0) and np.all(m.status() == 0)
    rel = np.linalg.norm(m.com() - b.com(), axis=1) / np.linalg.norm(b.com(), axis=1)
    assert np.all(rel <= 1e-5), rel


def test_dynamic_mix_batch_matches_oracle():
    """Eight seeded robots over pacemaker signals driving cilia, boundary-condition regions,
    attachment of Sticky materials and detach, in one FP64 batch: each follows the oracle
    (positions within 1e-6 voxel sizes, the same surface sets and runtime links)."""
    import feature_mix
    robots = [feature_mix.robot_dynamic(s) for s in range(8)]
    b = abi.Batch(robots, abi.PRECISION_FP64)
    sims = [ob.oracle_sim(r) for r in robots]
    off = b.voxel_offset
    for _ in range(4):
        b.step(60)
        pos, surf, used = b.state()["pos"], b.surface(), b.links_in_use()
        for i, (r, s) in enumerate(zip(robots, sims)):
            s.step(60)
            err = np.max(np.abs(_robot_slice(b, i, pos) - s.voxels()["pos"]))
            assert err <= POS_TOL * r.vox_size, f"robot {i}: {err:.3e}"
            mine = surf[(surf >= off[i]) & (surf < off[i + 1])] - off[i]
            assert np.array_equal(mine, s.surface()), f"robot {i}: surface"
            assert used[i] == s.counts()[1], f"robot {i}: links in use"
    assert np.all(b.status() == 0)


def test_models_mix_batch_matches_oracle():
    """Eight seeded robots mixing bilinear (plastic), data-point and linear materials with
    failure and Poisson's ratio, in one FP64 batch: each follows the oracle (positions
    within 1e-6 voxel sizes)."""
    import feature_mix
    robots = [feature_mix.robot_models(s) for s in range(8)]
    b = abi.Batch(robots, abi.PRECISION_FP64)
    sims = [ob.oracle_sim(r) for r in robots]
    for _ in range(4):
        b.step(60)
        pos = b.state()["pos"]
        for i, (r, s) in enumerate(zip(robots, sims)):
            s.step(60)
            err = np.max(np.abs(_robot_slice(b, i, pos) - s.voxels()["pos"]))
            assert err <= POS_TOL * r.vox_size, f"robot {i}: {err:.3e}"
    assert np.all(b.status() == 0)


def test_fp64_feature_mix_batch_matches_oracle():
    """Eight seeded robots combining collision, detach, material removal, cilia and
    force fields, in one batch: the FP64 kernels follow the oracle robot by robot
    (positions within 1e-6 voxel sizes, identical surface sets)."""
    import feature_mix
    robots = [feature_mix.robot(s) for s in range(8)]
    b = abi.Batch(robots, abi.PRECISION_FP64)
    sims = [ob.oracle_sim(r) for r in robots]
    off = b.voxel_offset
    for _ in range(4):
        b.step(60)
        pos, surf = b.state()["pos"], b.surface()
        for i, (r, s) in enumerate(zip(robots, sims)):
            s.step(60)
            err = np.max(np.abs(_robot_slice(b, i, pos) - s.voxels()["pos"]))
            assert err <= POS_TOL * r.vox_size, f"robot {i}: {err:.3e}"
            mine = surf[(surf >= off[i]) & (surf < off[i + 1])] - off[i]
            assert np.array_equal(mine, s.surface()), f"robot {i}: surface"
    assert np.all(b.status() == 0)
