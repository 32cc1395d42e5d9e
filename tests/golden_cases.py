"""Load the golden fixtures of tests/golden/ back into workloads.Robot objects."""

import glob
import json
import os

import numpy as np

from vx3g import workloads as wl

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load(name):
    d = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    s = json.loads(str(d["settings"]))
    tup = lambda n: tuple(tup(c) if isinstance(c, list) else c for c in n)  # noqa: E731
    for key in ("force_field", "attach_conditions"):  # math trees were stored as nested JSON lists
        if s.get(key) is not None:
            s[key] = [None if t is None else tup(t) for t in s[key]]
    mats = [wl.Material(E=m[0], nu=m[1], rho=m[2], cte=m[3], mu_static=m[4], mu_kinetic=m[5], fail_stress=m[6],
                        fixed=int(m[7]), is_measured=int(m[8]),
                        cilia=float(m[9]) if len(m) > 9 else 0.0, cilia_on_after=float(m[10]) if len(m) > 10 else 0.0,
                        remove_after=float(m[11]) if len(m) > 11 else 0.0, sticky=int(m[12]) if len(m) > 12 else 0,
                        thermal_on_after=float(m[13]) if len(m) > 13 else 0.0)
            for m in d["materials"]]
    if "models" in d.files:  # MatModel 2/3 parameters per palette entry
        for m, md in zip(mats, json.loads(str(d["models"]))):
            m.model = md["model"]
            m.plastic_mod = md["plastic_mod"]
            m.yield_stress = md["yield_stress"]
            m.ss_strain = None if md["ss_strain"] is None else tuple(md["ss_strain"])
            m.ss_stress = None if md["ss_stress"] is None else tuple(md["ss_stress"])
    if "signal_mats" in d.files:  # isPaceMaker, PaceMakerPeriod, signalValueDecay, signalTimeDelay, inactivePeriod
        for m, row in zip(mats, d["signal_mats"]):
            m.is_pacemaker, m.pacemaker_period, m.signal_value_decay, m.signal_time_delay, m.inactive_period = (
                int(row[0]), float(row[1]), float(row[2]), float(row[3]), float(row[4]))
    phase = d["phase"] if d["phase"].size else None
    robot = wl.Robot(grid=d["lattice"], materials=mats, phase=phase, z_offset=0, **s)
    if "bcs" in d.files:  # boundary-condition regions
        robot.bcs = [wl.BCRegion(**{k: tuple(v) if isinstance(v, list) else v for k, v in b.items()})
                     for b in json.loads(str(d["bcs"]))]
    for name in ("cilia_base", "cilia_shift"):
        if name in d.files and d[name].size:
            setattr(robot, name, d[name])
    return robot, d
