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
