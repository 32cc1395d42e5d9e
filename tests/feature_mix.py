"""Seeded random robots that combine every feature the oracle restates: thermal
actuation, self-collision, detach, material removal (SecondaryExperiment), cilia
and force fields (shared by the oracle and GPU parity tests)."""

import numpy as np

from vx3g import workloads as wl


def robot(seed):
    rng = np.random.default_rng(1000 + seed)
    nmat = int(rng.integers(1, 4))
    mats = []
    for k in range(nmat):
        mats.append(wl.Material(E=float(10 ** rng.uniform(4.5, 6.5)), nu=float(rng.choice([0.0, 0.35])),
                                cte=float(rng.choice([0.0, 0.01])), mu_static=float(rng.uniform(0.2, 1.0)),
                                mu_kinetic=float(rng.uniform(0.05, 0.2)),
                                fail_stress=float(rng.choice([0.0, 1500.0, 4000.0])),
                                cilia=float(rng.choice([0.0, 0.8, -0.5])),
                                remove_after=float(rng.choice([0.0, 0.0015])) if k else 0.0))
    dims = tuple(int(x) for x in rng.integers(3, 7, size=3))
    robot = wl.bernoulli_body(rng, dims, 0.85, mats, random_phase=True, temp_vary=True,
                              temp_amplitude=float(rng.uniform(10, 40)), enable_collision=bool(seed % 2 == 0),
                              enable_expansion=int(seed % 3 == 0), z_offset=int(rng.integers(0, 2)))
    robot.volume_effects = bool(seed % 4 != 1)
    robot.enable_detach = seed % 3 != 2
    robot.secondary_experiment = seed % 2 == 1 or seed == 4
    robot.enable_cilia = seed % 4 in (0, 3)
    if robot.enable_cilia:
        robot.cilia_base = 1e-2 * rng.standard_normal(robot.grid.shape + (3,))
    if seed % 3 == 1:
        C = lambda v: ("mtCONST", v)  # noqa: E731
        V = lambda n: ("mtVAR", n)  # noqa: E731
        robot.force_field = [("mtMUL", C(2e-3), ("mtSIN", ("mtMUL", C(40.0), V("t")))), None,
                             ("mtMUL", C(-0.2), ("mtSUB", V("z"), C(0.02)))]
    return robot


def robot_settings(seed):
    """Seeded random robots over the settings the fixed workloads leave at their defaults:
    densities, Poisson's ratios, CTEs, friction, isMeasured, thermal turn-on delays, Fixed
    voxels, lattice size, DtFrac, global/bond/collision damping, gravity, and a static
    temperature (TempEnabled without VaryTempEnabled) for the robots that do not actuate."""
    rng = np.random.default_rng(2000 + seed)
    nmat = int(rng.integers(2, 5))
    mats = []
    for k in range(nmat):
        mats.append(wl.Material(E=float(10 ** rng.uniform(4.5, 6.5)), nu=float(rng.choice([0.0, 0.2, 0.35, 0.45])),
                                rho=float(rng.choice([400.0, 1000.0, 2500.0])),
                                cte=float(rng.choice([0.0, 0.005, 0.01])), mu_static=float(rng.uniform(0.2, 1.0)),
                                mu_kinetic=float(rng.uniform(0.05, 0.3)), is_measured=int(rng.choice([1, 1, 0])),
                                thermal_on_after=float(rng.choice([0.0, 0.0, 0.002]))))
    vary = seed % 2 == 0
    dims = tuple(int(x) for x in rng.integers(3, 7, size=3))
    robot = wl.bernoulli_body(rng, dims, 0.85, mats, random_phase=True, temp_vary=vary,
                              temp_amplitude=float(rng.uniform(10, 40) if vary else rng.uniform(5, 25)),
                              enable_collision=seed % 4 < 2, enable_expansion=int(seed % 3 != 1),
                              z_offset=int(rng.integers(0, 2)))
    robot.temp_enabled = not vary
    robot.volume_effects = seed % 4 != 3
    robot.vox_size = float(rng.choice([0.005, 0.01, 0.02]))
    robot.dt_frac = float(rng.uniform(0.4, 0.95))
    robot.slow_damping = float(rng.choice([0.0, 0.02, 0.1]))
    robot.bond_damping = float(rng.uniform(0.3, 1.2))
    robot.col_damping = float(rng.uniform(0.5, 1.5))
    robot.grav_acc = float(rng.choice([-9.81, -4.0]))
    if seed % 3 == 0:  # one or two voxels of a Fixed material
        robot.materials = mats + [wl.Material(E=1e6, nu=0.35, fixed=1)]
        occ = np.argwhere(robot.grid > 0)
        for z, y, x in occ[rng.choice(len(occ), min(2, len(occ) - 1), replace=False)]:
            robot.grid[z, y, x] = len(robot.materials)
    return robot


def robot_dynamic(seed):
    """Seeded random robots over the run-time features together: pacemaker signals driving
    cilia, boundary-condition regions (fixed DOFs, forces, torques, displacements),
    attachment of Sticky materials, detach, on actuated, self-colliding bodies."""
    rng = np.random.default_rng(3000 + seed)
    sticky = seed % 2 == 0
    mats = [wl.Material(E=float(10 ** rng.uniform(5.0, 6.3)), nu=0.0 if sticky else 0.35, cte=0.01,
                        sticky=int(sticky), cilia=float(rng.choice([0.0, 0.6])),
                        fail_stress=float(rng.choice([0.0, 4000.0])) if not sticky else 0.0,
                        is_pacemaker=int(seed % 3 == 0), pacemaker_period=0.002,
                        mu_static=float(rng.uniform(0.3, 1.0)), mu_kinetic=float(rng.uniform(0.05, 0.3))),
            wl.Material(E=float(10 ** rng.uniform(5.0, 6.3)), nu=0.0, cte=float(rng.choice([0.0, 0.01])),
                        sticky=int(sticky), cilia=float(rng.choice([0.0, -0.4])))]
    dims = tuple(int(x) for x in rng.integers(4, 7, size=3))
    robot = wl.bernoulli_body(rng, dims, 0.8, mats, random_phase=True, temp_vary=True,
                              temp_amplitude=float(rng.uniform(20, 39)), enable_collision=True, enable_expansion=1,
                              z_offset=int(rng.integers(0, 2)))
    robot.volume_effects = not sticky
    robot.enable_attach = sticky
    robot.safety_guard = int(rng.choice([0, 20]))
    robot.enable_detach = not sticky
    robot.enable_signals = seed % 3 != 2
    robot.enable_cilia = True
    robot.cilia_base = 1e-2 * rng.standard_normal(robot.grid.shape + (3,))
    robot.cilia_shift = 5e-3 * rng.standard_normal(robot.grid.shape + (3,))
    if seed % 4 < 2:  # a fixed slab at one end, a pushed region at the other
        robot.bcs = [wl.BCRegion(prim=0, dof_fixed=int(rng.choice([7, 63])), x=0.0, y=0.0, z=0.0, dx=0.2, dy=1.0,
                                 dz=1.0),
                     wl.BCRegion(prim=0, dof_fixed=0, x=0.75, y=0.0, z=0.0, dx=0.25, dy=1.0, dz=1.0,
                                 force=(0.0, 0.0, float(rng.uniform(-0.05, 0.05))),
                                 torque=(float(rng.uniform(-1e-4, 1e-4)), 0.0, 0.0))]
    return robot


def robot_models(seed):
    """Seeded random robots mixing the stress-strain models: bilinear (elastic-plastic,
    with or without failure), data-point curves and linear materials (with or without
    failure), Poisson's ratio on or off, on actuated bodies, some self-colliding."""
    rng = np.random.default_rng(4000 + seed)
    nu = float(rng.choice([0.0, 0.3]))
    E1 = float(10 ** rng.uniform(4.8, 5.5))
    ys = float(rng.uniform(50.0, 200.0))
    bil = wl.Material(E=E1, nu=nu, cte=0.01, model=2, plastic_mod=E1 * float(rng.uniform(0.1, 0.5)),
                      yield_stress=ys, fail_stress=float(rng.choice([-1.0, 6.0 * ys])))
    s1 = float(rng.uniform(0.001, 0.003))
    s2, s3 = s1 * float(rng.uniform(2.0, 4.0)), 0.0
    s3 = s2 * float(rng.uniform(2.0, 4.0))
    k1 = float(10 ** rng.uniform(4.8, 5.3))
    f1 = k1 * s1
    f2 = f1 + 0.5 * k1 * (s2 - s1)
    f3 = f2 + 0.2 * k1 * (s3 - s2)
    dat = wl.Material(E=0, nu=nu, cte=0.01, model=3, ss_strain=(0.0, s1, s2, s3), ss_stress=(0.0, f1, f2, f3))
    lin = wl.Material(E=float(10 ** rng.uniform(4.8, 5.5)), nu=nu, cte=float(rng.choice([0.0, 0.01])),
                      fail_stress=float(rng.choice([0.0, 800.0])))
    dims = tuple(int(x) for x in rng.integers(4, 7, size=3))
    return wl.bernoulli_body(rng, dims, 0.85, [bil, dat, lin], random_phase=True, temp_vary=True,
                             temp_amplitude=float(rng.uniform(5.0, 12.0)), temp_period=0.02, enable_expansion=1,
                             enable_collision=seed % 2 == 0, z_offset=1, volume_effects=nu > 0 or seed % 3 == 0)
