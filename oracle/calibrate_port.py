"""Time the C restatement (oracle/_build/liboracle.so) against the reference's own step
compiled on the host (oracle/_ref/libvx3ref.so) on the same robots and steps, one host
thread each (TEST INFRASTRUCTURE: relates the CPU baseline and the reference arm of
bench.py, which time the restatement, to the reference's own code).

    make -C oracle oracle ref REF=<voxcraft-sim tree>
    python oracle/calibrate_port.py

Prints, per case, the seconds per step of each and the ratio reference / restatement.
"""

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
import oracle_bridge as ob  # noqa: E402
from vx3g import workloads as wl  # noqa: E402


def per_step(sim, steps):
    sim.step(2)  # the first step also sets the time step up
    t0 = time.perf_counter()
    done = sim.step(steps)
    return (time.perf_counter() - t0) / max(done, 1)


def cases():
    rng = np.random.default_rng(5)
    mats = [wl.Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, cte=0.01) for _ in range(4)]
    c3_like = wl.bernoulli_body(rng, (16, 16, 16), 0.7, mats, random_phase=True, temp_vary=True,
                                temp_amplitude=39.0)
    c5_like = wl.bernoulli_body(rng, (12, 12, 12), 0.65, mats, random_phase=True, temp_vary=True,
                                temp_amplitude=39.0, enable_collision=True, enable_expansion=1)
    return [("16^3 Bernoulli(0.7) body, 4 materials, actuation, no collisions (link + voxel passes)", c3_like, 200),
            ("12^3 Bernoulli(0.65) body, actuation, self-collision (whole steps, all-pairs loop)", c5_like, 40),
            ("10^3 block drop, floor (link + voxel passes)", wl.c1_block_drop()[0], 400)]


def main():
    if not ob.ref_available():
        sys.exit("reference build missing: run `make -C oracle ref` first")
    for name, robot, steps in cases():
        t_port = per_step(ob.oracle_sim(robot), steps)
        t_ref = per_step(ob.ref_sim(robot), steps)
        nv = ob.oracle_sim(robot).counts()[0]
        print(f"{name}: {nv} voxels, {steps} steps; restatement {t_port * 1e3:.3f} ms/step, "
              f"reference build {t_ref * 1e3:.3f} ms/step, ratio {t_ref / t_port:.2f}")


if __name__ == "__main__":
    main()
