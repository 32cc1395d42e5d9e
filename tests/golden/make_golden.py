"""Generate golden vectors from the reference's own VX3 physics (host build).

Run where the reference tree is mounted:

    make -C oracle ref            # compiles the reference sources into oracle/_ref/
    python tests/golden/make_golden.py [case ...]

Each case is a small seeded robot.  The VXA document is fed to the
reference's own reader (CXML_Rip + CVX_Sim::ReadVXA/Import) and stepped by the
reference's VX3_Link/VX3_Voxel/VX3_Collision code; snapshots of the state are
written to tests/golden/<case>.npz together with the inputs needed to rebuild
the same robot without the reference (lattice, phase, palette, settings).
The reference produces no golden vectors of its own for this path, so these
files are what pins the oracle and, through it, the GB300 kernels.
"""

import dataclasses
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
import vx3g.workloads as wl  # noqa: E402
import oracle_bridge as ob  # noqa: E402


def cases():
    """name -> (robot, steps, snapshot every)"""
    out = {}
    out["block3_drop"] = (wl.solid_block(3), 600, 200)
    out["block10_drop"] = (wl.solid_block(10), 200, 100)
    rng = np.random.default_rng(1)
    mats = [wl.Material(E=1e6, nu=0.35, cte=0.0), wl.Material(E=1e6, nu=0.35, cte=0.01)]
    out["bern6_thermal_collision"] = (
        wl.bernoulli_body(rng, (6, 6, 6), 0.6, mats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                          temp_period=0.2, enable_collision=True, enable_expansion=1, z_offset=1), 400, 100)
    rng = np.random.default_rng(2)
    mats4 = [wl.Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, cte=0.01) for _ in range(4)]
    out["bern8_4mat_phase"] = (
        wl.bernoulli_body(rng, (8, 7, 5), 0.7, mats4, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                          temp_period=0.2, z_offset=0), 300, 100)
    soft = [wl.Material(E=2e4, nu=0.0, rho=1e3, mu_static=0.2, mu_kinetic=0.1)]
    grid = np.zeros((3, 2, 9), np.uint8)
    grid[2, :, :] = 1        # a thin overhanging sheet ...
    grid[:, :, 0:2] = 1      # ... on a short pillar: the free end sags into the large-angle branch
    out["soft_cantilever_large_angle"] = (wl.Robot(grid=grid, materials=soft, volume_effects=False, z_offset=0),
                                          1500, 500)
    brittle = [wl.Material(E=2e4, nu=0.0, fail_stress=40.0, mu_static=0.2, mu_kinetic=0.1)]
    out["brittle_failure"] = (wl.Robot(grid=grid.copy(), materials=brittle, volume_effects=False, z_offset=0),
                              900, 300)
    # Simulator/ForceField programs (VX3_Voxel.cu:178-184): time, position and voxel-count terms
    C = lambda v: ("mtCONST", v)  # noqa: E731
    V = lambda n: ("mtVAR", n)  # noqa: E731
    ff = [("mtMUL", C(1e-2), ("mtSIN", ("mtMUL", C(31.4), V("t")))),
          ("mtSUB", ("mtMUL", C(-0.5), V("y")), ("mtDIV", V("num_voxel"), C(1e5))),
          ("mtADD", ("mtMUL", C(6e-3), ("mtNORMALCDF", ("mtDIV", ("mtSUB", V("z"), C(0.02)), C(0.01)))),
                    ("mtMUL", C(2e-3), ("mtATAN", ("mtPOW", ("mtMUL", V("t"), C(10.0)), C(2.0)))))]
    ffmats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=3e5, nu=0.35, cte=0.0)]
    rng = np.random.default_rng(7)
    out["bern5_force_field"] = (
        wl.bernoulli_body(rng, (5, 4, 3), 0.8, ffmats, random_phase=True, temp_vary=True, temp_amplitude=20.0,
                          force_field=ff, z_offset=1), 300, 100)
    # TurnOnThermalExpansionAfterThisManySeconds: two of three actuated materials start
    # expanding later, at about step 129 and step 241 (dt = 2.49e-5 s)
    rng = np.random.default_rng(17)
    tmats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=5e5, nu=0.35, cte=0.01, thermal_on_after=0.0032),
             wl.Material(E=8e5, nu=0.35, cte=0.008, thermal_on_after=0.006)]
    out["bern5_thermal_delay"] = (
        wl.bernoulli_body(rng, (5, 5, 4), 0.8, tmats, random_phase=True, temp_vary=True, temp_amplitude=30.0,
                          enable_expansion=1, z_offset=1), 300, 100)
    # Thermal/TempEnabled without VaryTempEnabled: every voxel starts at TempBase + TempAmplitude, so
    # one material of a two-material block is expanded by 20% from the start (a bimetal that bends
    # as it drops)
    smats = [wl.Material(E=5e5, nu=0.35, cte=0.01), wl.Material(E=5e5, nu=0.35, cte=0.0)]
    sgrid = np.ones((3, 4, 6), np.uint8)
    sgrid[:, :2, :] = 2
    out["bimetal_static_expansion"] = (
        wl.Robot(grid=sgrid, materials=smats, temp_enabled=True, temp_amplitude=20.0, enable_expansion=1,
                 z_offset=1), 300, 100)
    # Settings every other case leaves at their defaults: global (slow) damping, bond and
    # collision damping other than 1, DtFrac 0.5 and a weaker gravity, on an actuated,
    # self-colliding body
    rng = np.random.default_rng(19)
    dmats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=3e5, nu=0.3, cte=0.005, mu_static=0.6,
                                                                mu_kinetic=0.3)]
    dmp = wl.bernoulli_body(rng, (6, 5, 4), 0.75, dmats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                            enable_collision=True, enable_expansion=1, z_offset=1)
    dmp.slow_damping, dmp.bond_damping, dmp.col_damping, dmp.dt_frac, dmp.grav_acc = 0.05, 0.4, 0.7, 0.5, -5.0
    out["bern6_damping_settings"] = (dmp, 300, 100)
    # Material properties every other case leaves alike: densities 400 and 2500 kg/m^3,
    # Poisson's ratios 0.45 and 0.2, a material left out of the centre of mass (isMeasured 0)
    # and a Fixed one, on an actuated, self-colliding body
    rng = np.random.default_rng(23)
    pmats = [wl.Material(E=6e5, nu=0.45, rho=400.0, cte=0.01),
             wl.Material(E=2e6, nu=0.2, rho=2500.0, cte=0.004, is_measured=0),
             wl.Material(E=1e6, nu=0.35, rho=1500.0, cte=0.008),
             wl.Material(E=1e6, nu=0.35, fixed=1)]
    pg = wl.bernoulli_body(rng, (6, 5, 4), 0.8, pmats[:3], random_phase=True, temp_vary=True, temp_amplitude=39.0,
                           enable_collision=True, enable_expansion=1, z_offset=1)
    occ = np.argwhere(pg.grid[1:] > 0)  # two voxels above the body's bottom layer held Fixed
    for z, y, x in occ[rng.choice(len(occ), 2, replace=False)]:
        pg.grid[z + 1, y, x] = 4
    pg.materials = pmats
    out["bern6_density_measured_fixed"] = (pg, 300, 100)
    # A robot of one voxel (no links: the time step from the voxel's own stiffness), actuated,
    # dropped onto the floor, where it sticks and slips as it breathes
    one = wl.Robot(grid=np.ones((1, 1, 1), np.uint8), materials=[wl.Material(E=1e6, nu=0.35, cte=0.01,
                                                                             mu_static=0.4, mu_kinetic=0.2)],
                   phase=np.full((1, 1, 1), 0.3), temp_vary=True, temp_amplitude=39.0, enable_expansion=1,
                   z_offset=1)
    out["voxel1_actuated_drop"] = (one, 1500, 500)
    # A lattice of 2.5 cm voxels (every other case uses 1 cm): masses, stiffnesses, the
    # collision cutoff and the floor scale with it
    rng = np.random.default_rng(29)
    vmats = [wl.Material(E=1e6, nu=0.35, cte=0.01), wl.Material(E=4e5, nu=0.35, cte=0.01)]
    big = wl.bernoulli_body(rng, (5, 5, 4), 0.8, vmats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                            enable_collision=True, enable_expansion=1, z_offset=1)
    big.vox_size = 0.025
    out["bern5_voxsize_25mm"] = (big, 300, 100)
    # Link failure with Poisson's ratio (the failure stress of the volume-effects model) and
    # detach: an actuated block whose softer links fail and leave the lattice
    rng = np.random.default_rng(31)
    fmats = [wl.Material(E=2e5, nu=0.3, fail_stress=3000.0, cte=0.01, mu_static=0.3, mu_kinetic=0.2),
             wl.Material(E=6e5, nu=0.4, cte=0.005)]
    fb = wl.bernoulli_body(rng, (4, 4, 4), 1.0, fmats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                           enable_collision=True, enable_expansion=1, z_offset=0)
    fb.enable_detach = True
    out["block4_fail_poisson_detach"] = (fb, 300, 100)
    # EnableCilia: per-voxel BaseCiliaForce/ShiftCiliaForce, a negative Cilia and a turn-on time
    rng = np.random.default_rng(9)
    cmats = [wl.Material(E=1e6, nu=0.35, cte=0.01, cilia=1.0),
             wl.Material(E=3e5, nu=0.35, cilia=-0.5, cilia_on_after=0.003), wl.Material(E=5e5, nu=0.35)]
    cil = wl.bernoulli_body(rng, (5, 4, 3), 0.85, cmats, random_phase=True, temp_vary=True, temp_amplitude=20.0,
                            z_offset=1)
    cil.enable_cilia = True
    cil.cilia_base = 2e-2 * rng.standard_normal(cil.grid.shape + (3,))
    cil.cilia_shift = 1e-2 * rng.standard_normal(cil.grid.shape + (3,))
    out["bern5_cilia"] = (cil, 300, 100)
    # EnableDetach: a brittle, thermally driven block; links fail in the first steps, interior
    # voxels become surface voxels and the loose pieces collide
    rng = np.random.default_rng(6)
    bmats = [wl.Material(E=1e5, nu=0.0, fail_stress=2500.0, mu_static=0.2, mu_kinetic=0.1, cte=0.001)]
    out["block4_detach"] = (wl.Robot(grid=np.ones((4, 4, 4), np.uint8), materials=bmats, volume_effects=False,
                                     z_offset=0, enable_collision=True, enable_detach=True,
                                     phase=rng.random((4, 4, 4)), temp_vary=True, temp_amplitude=30.0,
                                     enable_expansion=1), 300, 100)
    # detach with cilia: voxels exposed by failed links get cilia forces from the step after
    rng = np.random.default_rng(13)
    dcm = [wl.Material(E=1e5, nu=0.0, fail_stress=2500.0, mu_static=0.2, mu_kinetic=0.1, cte=0.001, cilia=0.8)]
    dc = wl.Robot(grid=np.ones((4, 4, 4), np.uint8), materials=dcm, volume_effects=False, z_offset=0,
                  enable_collision=True, enable_detach=True, phase=rng.random((4, 4, 4)), temp_vary=True,
                  temp_amplitude=30.0, enable_expansion=1, enable_cilia=True)
    dc.cilia_base = 1e-2 * rng.standard_normal((4, 4, 4, 3))
    out["block4_detach_cilia"] = (dc, 300, 100)
    # SecondaryExperiment: two materials leave the simulation at different times; the
    # exposed voxels join the collision surface and, with cilia on, get cilia forces
    rng = np.random.default_rng(11)
    rmats = [wl.Material(E=1e6, nu=0.35, cte=0.01, cilia=1.0),
             wl.Material(E=3e5, nu=0.35, remove_after=0.002),
             wl.Material(E=5e5, nu=0.35, cilia=-0.5, remove_after=0.006)]
    rem = wl.bernoulli_body(rng, (6, 5, 4), 0.9, rmats, random_phase=True, temp_vary=True, temp_amplitude=20.0,
                            enable_collision=True, z_offset=1)
    rem.enable_cilia = True
    rem.secondary_experiment = True
    rem.cilia_base = 2e-2 * rng.standard_normal(rem.grid.shape + (3,))
    out["bern6_removal"] = (rem, 300, 100)
    # bilinear (elastic-plastic) overhang clamped at the base (a Fixed material, floor off,
    # so no stick/slip): gravity loads the root links past yield, the oscillation then
    # unloads them along the offset line (VX3_Link::updateStrain)
    plastic = [wl.Material(E=2e4, nu=0.0, rho=1e3, model=2, plastic_mod=4e3, yield_stress=8.0, fail_stress=-1.0),
               wl.Material(E=2e4, nu=0.0, rho=1e3, fixed=1)]
    clamp = grid.copy()
    clamp[0, :, 0:2] = 2
    out["bilinear_cantilever_plastic"] = (wl.Robot(grid=clamp, materials=plastic, volume_effects=False,
                                                   z_offset=0, floor=False), 1500, 500)
    # actuated body mixing a bilinear material with failure, a data-point curve and a
    # linear material (merged link curves, springs in series), Poisson's ratio off
    rng = np.random.default_rng(4)
    dat = wl.Material(E=0, nu=0.0, cte=0.01, model=3, ss_strain=(0, 0.002, 0.006, 0.02, 0.05),
                      ss_stress=(0, 200.0, 450.0, 700.0, 800.0))
    bil = wl.Material(E=1e5, nu=0.0, cte=0.01, model=2, plastic_mod=3e4, yield_stress=100.0, fail_stress=900.0)
    out["bern5_data_bilinear"] = (
        wl.bernoulli_body(rng, (5, 4, 3), 0.9, [bil, dat, wl.Material(E=1e5, nu=0.0)], random_phase=True,
                          temp_vary=True, temp_amplitude=8.0, temp_period=0.02, enable_expansion=1, z_offset=1,
                          volume_effects=False), 400, 100)
    # the same with Poisson's ratio on: the volumetric variant of the non-linear stress
    rng = np.random.default_rng(5)
    datnu = wl.Material(E=0, nu=0.3, cte=0.01, model=3, ss_strain=(0.002, 0.006, 0.02), ss_stress=(200.0, 450.0, 600.0))
    bilnu = wl.Material(E=1e5, nu=0.35, cte=0.01, model=2, plastic_mod=2e4, yield_stress=150.0, fail_stress=-1.0)
    out["bern4_data_bilinear_poisson"] = (
        wl.bernoulli_body(rng, (4, 4, 4), 0.9, [datnu, bilnu, wl.Material(E=1e5, nu=0.3, cte=0.0)],
                          random_phase=True, temp_vary=True, temp_amplitude=8.0, temp_period=0.02,
                          enable_expansion=1, z_offset=1), 400, 100)
    # boundary conditions: a cantilever clamped (all six DOFs) on its first layer with a
    # load on its last, floor off
    beam_bcs = [wl.BCRegion(prim=0, dof_fixed=63, x=0.0, y=0.0, z=0.0, dx=0.05, dy=1.0, dz=1.0),
                wl.BCRegion(prim=0, dof_fixed=0, x=0.95, y=0.0, z=0.0, dx=0.05, dy=1.0, dz=1.0, force=(0.0, 0.0, -0.02))]
    out["beam10_clamped_bcs"] = (wl.Robot(grid=np.ones((2, 2, 10), np.uint8), materials=[wl.Material(E=1e5, nu=0.35)],
                                          floor=False, bcs=beam_bcs), 600, 200)
    # partial DOFs on an actuated body on the floor: X/Y translation (with a displacement)
    # and the Z rotation held on one face, a sphere region with a force and a torque, a
    # cylinder fixing the X rotation, a box fixing Z translation and Y rotation; regions
    # overlap (the reference's force accumulation doubles earlier shares)
    rng = np.random.default_rng(21)
    bmats = [wl.Material(E=2e5, nu=0.35, cte=0.01), wl.Material(E=1e5, nu=0.35)]
    part = wl.bernoulli_body(rng, (6, 5, 4), 0.9, bmats, random_phase=True, temp_vary=True, temp_amplitude=15.0,
                             temp_period=0.05, z_offset=0)
    part.bcs = [wl.BCRegion(prim=0, dof_fixed=1 | 2 | 32, x=0.0, y=0.0, z=0.0, dx=0.2, dy=1.0, dz=1.0,
                            displace=(0.001, 0.0, 0.0), ang_displace=(0.0, 0.0, 0.05)),
                wl.BCRegion(prim=2, dof_fixed=0, x=0.7, y=0.5, z=0.6, radius=0.2, torque=(1e-4, 0.0, 2e-4),
                            force=(0.0, 0.01, 0.0)),
                wl.BCRegion(prim=1, dof_fixed=8, x=0.0, y=0.5, z=0.5, dx=1.0, radius=0.15, force=(0.0, 0.0, 0.005)),
                wl.BCRegion(prim=0, dof_fixed=4 | 16, x=0.5, y=0.0, z=0.0, dx=0.5, dy=0.5, dz=0.3,
                            displace=(0.0, 0.0, -0.0005), force=(0.003, 0.0, 0.0))]
    out["bern6_partial_bcs"] = (part, 400, 100)
    # EnableSignals: pacemaker voxels fire every 2 ms, signals spread along links with short
    # delays and decay; each voxel's signal scales its ShiftCiliaForce; self-collision on
    rng = np.random.default_rng(17)
    smats = [wl.Material(E=1e6, nu=0.35, cte=0.01, cilia=1.0, signal_time_delay=0.0004, inactive_period=0.0006),
             wl.Material(E=3e5, nu=0.35, is_pacemaker=1, pacemaker_period=0.002, signal_time_delay=0.0003,
                         inactive_period=0.0005, signal_value_decay=0.95, cilia=0.5),
             wl.Material(E=5e5, nu=0.35, cilia=-0.8, signal_time_delay=0.0002, inactive_period=0.0004,
                         signal_value_decay=0.85)]
    sig = wl.bernoulli_body(rng, (6, 5, 4), 0.85, smats, random_phase=True, temp_vary=True, temp_amplitude=15.0,
                            z_offset=1, enable_collision=True)
    sig.enable_cilia = True
    sig.enable_signals = True
    sig.cilia_base = 1e-2 * rng.standard_normal(sig.grid.shape + (3,))
    sig.cilia_shift = 2e-4 * rng.standard_normal(sig.grid.shape + (3,))
    out["bern6_signals_cilia"] = (sig, 400, 100)
    # EnableAttach: sticky pieces dropped on a sticky plate link up where they land (Z axis),
    # each far (over five links) from the other; a piece of another sticky material and a
    # non-sticky piece only collide; the first condition holds attachment off for 4 ms and
    # SafetyGuard 60 ends the new links' force scaling within the run
    att = np.zeros((5, 3, 11), np.uint8)
    att[0, :, :] = 1
    att[2:4, 1, 0:2] = 1
    att[2:4, 1, 4:6] = 1
    att[2:4, 1, 8] = 2
    att[2, 0:2, 10] = 3
    amats = [wl.Material(E=1e5, nu=0.0, sticky=1, mu_static=0.5, mu_kinetic=0.3),
             wl.Material(E=2e5, nu=0.0, sticky=1), wl.Material(E=1e5, nu=0.0)]
    out["sticky_drop_attach"] = (wl.Robot(grid=att, materials=amats, volume_effects=False, enable_collision=True,
                                          enable_attach=True, safety_guard=60,
                                          attach_conditions=[("mtGREATERTHAN", ("mtVAR", "t"), ("mtCONST", 0.004))]),
                                 800, 200)
    # three bimorph U shapes (each arm an expanding outer layer on a passive inner one, so the
    # arms bend together as the temperature rises) facing x, y and z: their tips touch and
    # link along all three axes, ten links at five-link spacing (floor off; no stick/slip,
    # so the run is not chaotic: a 1e-12 m nudge stays below 1e-9 m over the run)
    arm, w = 8, 5
    L = arm + 1
    u = np.zeros((L, 2 * w + 3, w + L + 2), np.uint8)
    u[0, 0, 0:w] = 2
    u[1:L, 0, 0] = 1
    u[1:L, 0, 1] = 2
    u[1:L, 0, w - 1] = 1
    u[1:L, 0, w - 2] = 2
    y0, x0 = 2, w + 2
    u[0, y0:y0 + w, 3] = 2
    u[1:L, y0, 3] = 1
    u[1:L, y0 + 1, 3] = 2
    u[1:L, y0 + w - 1, 3] = 1
    u[1:L, y0 + w - 2, 3] = 2
    u[0:w, y0, x0] = 2
    u[0, y0, x0:x0 + L] = 1
    u[1, y0, x0 + 1:x0 + L] = 2
    u[w - 1, y0, x0:x0 + L] = 1
    u[w - 2, y0, x0 + 1:x0 + L] = 2
    umats = [wl.Material(E=1e5, nu=0.0, sticky=1, cte=0.01), wl.Material(E=1e5, nu=0.0, sticky=1, cte=0.0)]
    out["bimorph_u3_attach"] = (wl.Robot(grid=u, materials=umats, volume_effects=False, enable_collision=True,
                                         enable_attach=True, temp_vary=True, temp_amplitude=20.0, temp_period=0.05,
                                         enable_expansion=1, floor=False, safety_guard=40, phase=np.zeros(u.shape),
                                         attach_conditions=[("mtGREATERTHAN", ("mtVAR", "t"), ("mtCONST", 0.002)),
                                                            None, ("mtLESSTHAN", ("mtVAR", "z"), ("mtCONST", 1.0))]),
                                1600, 400)
    return out


def snapshot(s, plastic=False, signals=False, attach=0):
    v = s.voxels()
    lk = s.links()
    t = s.topology()
    out = dict(small=t["small"], states=t["states"], pos=v["pos"], orient=v["orient"], linmom=v["linmom"], angmom=v["angmom"], tempe=v["tempe"],
               flags=v["flags"], strain=lk["strain"], maxstrain=lk["maxstrain"], rest=lk["rest"],
               local9=lk["local9"], forces=lk["forces"], contact=s.last_contact(), com=s.com(),
               time=np.array([s.time()]), dt=np.array([s.dt()], np.float32))
    if plastic:  # non-linear materials: the links' plastic strain offsets
        out["soffset"] = s.link_offsets()
    if signals:  # EnableSignals: every voxel's localSignal
        out["signal"] = s.signals()
    if attach:  # EnableAttach (attach = the palette size): the link table as it stands, runtime links appended
        out["negpos"], out["axis"], out["slots"] = t["negpos"], t["axis"], t["slots"]
        out["lmat_of_link"] = s.materials(attach)["lmat_of_link"]
    return out


def nonlinear(r):
    return any(m.mat_model() >= 2 for m in r.materials)


def robot_record(r):
    g, ph = r.padded()
    mats = np.array([[m.E, m.nu, m.rho, m.cte, m.mu_static, m.mu_kinetic, m.fail_stress, m.fixed, m.is_measured,
                      m.cilia, m.cilia_on_after, m.remove_after, m.sticky, m.thermal_on_after] for m in r.materials],
                    np.float64)
    settings = dict(vox_size=r.vox_size, dt_frac=r.dt_frac, bond_damping=r.bond_damping, col_damping=r.col_damping,
                    slow_damping=r.slow_damping, gravity=r.gravity, grav_acc=r.grav_acc, floor=r.floor,
                    temp_vary=r.temp_vary, temp_amplitude=r.temp_amplitude, temp_period=r.temp_period,
                    temp_base=r.temp_base, temp_enabled=r.temp_enabled, enable_expansion=r.enable_expansion,
                    enable_collision=r.enable_collision,
                    volume_effects=r.volume_effects, force_field=r.force_field, enable_cilia=r.enable_cilia,
                    enable_detach=r.enable_detach, secondary_experiment=r.secondary_experiment,
                    enable_signals=r.enable_signals, enable_attach=r.enable_attach, safety_guard=r.safety_guard,
                    attach_conditions=r.attach_conditions)
    rec = dict(lattice=g, phase=(ph if ph is not None else np.zeros(0)), materials=mats,
               settings=np.array(json.dumps(settings)))
    if r.enable_signals:  # signal parameters per palette entry
        rec["signal_mats"] = np.array([[m.is_pacemaker, m.pacemaker_period, m.signal_value_decay, m.signal_time_delay,
                                        m.inactive_period] for m in r.materials], np.float64)
    if r.bcs:  # boundary-condition regions
        rec["bcs"] = np.array(json.dumps([dataclasses.asdict(b) for b in r.bcs]))
    if nonlinear(r):  # material models beyond linear: MatModel and its parameters per palette entry
        rec["models"] = np.array(json.dumps([dict(model=m.mat_model(), plastic_mod=m.plastic_mod,
                                                  yield_stress=m.yield_stress,
                                                  ss_strain=None if m.ss_strain is None else list(m.ss_strain),
                                                  ss_stress=None if m.ss_stress is None else list(m.ss_stress))
                                             for m in r.materials]))
    for name in ("cilia_base", "cilia_shift"):  # per cell of the padded lattice, 3 values each
        a = r.padded_cells(getattr(r, name))
        rec[name] = a.reshape(g.shape + (3,)) if a is not None else np.zeros(0)
    return rec


def main(only=()):
    if not ob.ref_available():
        sys.exit("reference build missing: run `make -C oracle ref` first")
    for name, (robot, steps, every) in cases().items():
        if only and name not in only:
            continue
        s = ob.ref_sim(robot)
        nv, nl, _ = s.counts()
        rec = robot_record(robot)
        topo = s.topology()
        mats = s.materials(len(robot.materials))
        rec.update({"topo_" + k: v for k, v in topo.items()})
        rec.update({"mat_" + k: v for k, v in mats.items()})
        rec["recommended_dt0"] = np.array([s.recommended_dt()])
        if nonlinear(robot):
            curves = s.link_curves()
            rec["link_curve_n"] = np.array([len(c) for c in curves], np.int32)
            rec["link_curves"] = np.concatenate(curves) if curves else np.zeros((0, 2), np.float32)
        done, snaps = 0, []
        while done < steps:
            n = s.step(every)
            done += every
            snaps.append(done)
            for k, v in snapshot(s, nonlinear(robot), robot.enable_signals,
                                 len(robot.materials) if robot.enable_attach else 0).items():
                rec[f"s{done}_{k}"] = v
            rec[f"s{done}_surface"] = s.surface()
            if n < every:
                break
        rec["snap_steps"] = np.array(snaps)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
        print(f"{name}: nv={nv} nl={nl} snaps={snaps} t={s.time():.6g} com={s.com()}")


if __name__ == "__main__":
    main(sys.argv[1:])  # optional case names: regenerate only those
