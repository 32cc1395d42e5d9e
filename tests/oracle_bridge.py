"""ctypes bridge to the two CPU checkers (test infrastructure).

* the C restatement  oracle/_build/liboracle.so  (built from oracle/vx3_oracle.c)
* the reference build oracle/_ref/libvx3ref.so   (built from the reference
  sources; only present where the reference tree is mounted)

Both expose the same getters, so a test can run the same synthetic robot
through either and compare arrays.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libvx3ref.so")


class VxoMaterial(ctypes.Structure):
    _fields_ = [("E", ctypes.c_double), ("nu", ctypes.c_double), ("rho", ctypes.c_double),
                ("cte", ctypes.c_double), ("mu_static", ctypes.c_double), ("mu_kinetic", ctypes.c_double),
                ("fail_stress", ctypes.c_double), ("model", ctypes.c_int), ("fixed", ctypes.c_int),
                ("is_measured", ctypes.c_int), ("thermal_on_after", ctypes.c_double),
                ("cilia", ctypes.c_double), ("cilia_on_after", ctypes.c_double), ("remove_after", ctypes.c_double),
                ("plastic_mod", ctypes.c_double), ("yield_stress", ctypes.c_double), ("n_data", ctypes.c_int),
                ("strain_data", ctypes.c_void_p), ("stress_data", ctypes.c_void_p),
                ("is_pacemaker", ctypes.c_int), ("pacemaker_period", ctypes.c_double),
                ("signal_value_decay", ctypes.c_double), ("signal_time_delay", ctypes.c_double),
                ("inactive_period", ctypes.c_double), ("sticky", ctypes.c_int)]


class VxoBC(ctypes.Structure):
    _fields_ = [("prim", ctypes.c_int), ("dof_fixed", ctypes.c_int), ("x", ctypes.c_float), ("y", ctypes.c_float),
                ("z", ctypes.c_float), ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
                ("radius", ctypes.c_float), ("force", ctypes.c_double * 3), ("torque", ctypes.c_double * 3),
                ("displace", ctypes.c_double * 3), ("ang_displace", ctypes.c_double * 3)]


class VxoRobot(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("lattice", ctypes.c_void_p), ("phase", ctypes.c_void_p),
                ("n_materials", ctypes.c_int), ("materials", ctypes.POINTER(VxoMaterial)),
                ("vox_size", ctypes.c_double), ("dt_frac", ctypes.c_double), ("grav_acc", ctypes.c_double),
                ("floor_enabled", ctypes.c_int),
                ("temp_amplitude", ctypes.c_double), ("temp_period", ctypes.c_double), ("temp_base", ctypes.c_double),
                ("temp_enabled", ctypes.c_int), ("vary_temp", ctypes.c_int), ("enable_expansion", ctypes.c_int),
                ("enable_collision", ctypes.c_int), ("volume_effects", ctypes.c_int),
                ("bond_damping", ctypes.c_double), ("col_damping", ctypes.c_double), ("slow_damping", ctypes.c_double),
                ("force_field", ctypes.c_void_p * 3),
                ("enable_cilia", ctypes.c_int), ("cilia_base", ctypes.c_void_p), ("cilia_shift", ctypes.c_void_p),
                ("enable_detach", ctypes.c_int), ("secondary_experiment", ctypes.c_int),
                ("n_bcs", ctypes.c_int), ("bcs", ctypes.POINTER(VxoBC)), ("enable_signals", ctypes.c_int),
                ("enable_attach", ctypes.c_int), ("safety_guard", ctypes.c_int), ("attach_cond", ctypes.c_void_p * 5)]


def build_oracle():
    if not os.path.exists(ORACLE_SO):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "oracle"])
    return ORACLE_SO


def _P(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _setup(lib, prefix):
    h = ctypes.c_void_p
    for name, res, args in [
        ("destroy", None, [h]),
        ("counts", None, [h, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
        ("step", ctypes.c_int, [h, ctypes.c_int]),
        ("time", ctypes.c_double, [h]),
        ("dt", ctypes.c_float, [h]),
        ("voxels", None, [h] + [ctypes.c_void_p] * 6),
        ("topology", None, [h] + [ctypes.c_void_p] * 3),
        ("link_topology", None, [h] + [ctypes.c_void_p] * 4),
        ("links", None, [h] + [ctypes.c_void_p] * 5),
        ("voxel_mats", None, [h] + [ctypes.c_void_p] * 3),
        ("link_mats", None, [h] + [ctypes.c_void_p] * 2),
        ("num_link_mats", ctypes.c_int, [h]),
        ("surface", None, [h, ctypes.c_void_p]),
        ("last_contact", None, [h, ctypes.c_void_p]),
        ("com", None, [h, ctypes.c_void_p]),
        ("recommended_dt", ctypes.c_double, [h]),
        ("link_offsets", None, [h, ctypes.c_void_p]),
        ("link_curve", ctypes.c_int, [h, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    ]:
        f = getattr(lib, prefix + name)
        f.restype = res
        f.argtypes = args
    return lib


class Sim:
    """A robot running on one of the CPU checkers; same getters for both."""

    def __init__(self, lib, prefix, handle, keep):
        self.lib, self.p, self.h, self._keep = lib, prefix, ctypes.c_void_p(handle), keep

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    def counts(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._f("counts")(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def step(self, n):
        return self._f("step")(self.h, n)

    # timing helpers of the C restatement (CPU baseline only)
    def step_no_collision(self, n):
        f = self.lib.vxo_step_no_collision
        f.restype, f.argtypes = ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]
        return f(self.h, n)

    def set_threads(self, n):
        f = self.lib.vxo_set_threads
        f.restype, f.argtypes = None, [ctypes.c_void_p, ctypes.c_int]
        f(self.h, n)

    def set_state(self, pos, orient, linmom, angmom, t, tempe, static_flag, local9, strain, maxstrain, link_flags):
        """Continue a run taken elsewhere: voxel state, time, temperatures, static friction,
        link state (link_flags bit 0 smallAngle, bit 2 LOCAL_VELOCITY_VALID)."""
        c = lambda a, t_: np.ascontiguousarray(a, t_)  # noqa: E731
        arrs = [c(pos, np.float64), c(orient, np.float64), c(linmom, np.float64), c(angmom, np.float64)]
        f = self.lib.vxo_set_voxels
        f.restype, f.argtypes = None, [ctypes.c_void_p] * 5
        f(self.h, *[_P(a) for a in arrs])
        more = [c(tempe, np.float32), c(static_flag, np.int32), c(local9, np.float64), c(strain, np.float32),
                c(maxstrain, np.float32), c(link_flags, np.int32)]
        g = self.lib.vxo_set_run_state
        g.restype, g.argtypes = None, [ctypes.c_void_p, ctypes.c_double] + [ctypes.c_void_p] * 6
        g(self.h, float(t), *[_P(a) for a in more])

    def set_exact_threads(self, n):
        """Run the C restatement on n threads with results identical to the serial step."""
        f = self.lib.vxo_set_exact_threads
        f.restype, f.argtypes = None, [ctypes.c_void_p, ctypes.c_int]
        f(self.h, n)

    def time_collision_rows(self, begin, end):
        f = self.lib.vxo_time_collision_rows
        f.restype, f.argtypes = ctypes.c_double, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        return f(self.h, begin, end)

    def time(self):
        return self._f("time")(self.h)

    def dt(self):
        return self._f("dt")(self.h)

    def recommended_dt(self):
        return self._f("recommended_dt")(self.h)

    def voxels(self):
        nv = self.counts()[0]
        pos, lm, am = np.zeros((nv, 3)), np.zeros((nv, 3)), np.zeros((nv, 3))
        orient = np.zeros((nv, 4))
        tempe = np.zeros(nv, np.float32)
        flags = np.zeros(nv, np.int32)
        self._f("voxels")(self.h, _P(pos), _P(orient), _P(lm), _P(am), _P(tempe), _P(flags))
        return dict(pos=pos, orient=orient, linmom=lm, angmom=am, tempe=tempe, flags=flags)

    def topology(self):
        nv, nl, _ = self.counts()
        mat = np.zeros(nv, np.int32)
        ijk = np.zeros((nv, 3), np.int32)
        slots = np.zeros((nv, 6), np.int32)
        self._f("topology")(self.h, _P(mat), _P(ijk), _P(slots))
        negpos = np.zeros((nl, 2), np.int32)
        axis, small, states = (np.zeros(nl, np.int32) for _ in range(3))
        self._f("link_topology")(self.h, _P(negpos), _P(axis), _P(small), _P(states))
        return dict(mat=mat, ijk=ijk, slots=slots, negpos=negpos, axis=axis, small=small, states=states)

    def links(self):
        nl = self.counts()[1]
        strain, maxstrain = np.zeros(nl, np.float32), np.zeros(nl, np.float32)
        rest = np.zeros(nl)
        local9 = np.zeros((nl, 9))
        forces = np.zeros((nl, 12))
        self._f("links")(self.h, _P(strain), _P(maxstrain), _P(rest), _P(local9), _P(forces))
        return dict(strain=strain, maxstrain=maxstrain, rest=rest, local9=local9, forces=forces)

    def materials(self, n_voxel_mats):
        f = np.zeros((n_voxel_mats, 16), np.float32)
        ns = np.zeros(n_voxel_mats)
        fm = np.zeros((n_voxel_mats, 2), np.int32)
        self._f("voxel_mats")(self.h, _P(f), _P(ns), _P(fm))
        nlm = self._f("num_link_mats")(self.h)
        lf = np.zeros((max(nlm, 1), 16), np.float32)
        lol = np.zeros(max(self.counts()[1], 1), np.int32)
        self._f("link_mats")(self.h, _P(lf), _P(lol))
        return dict(vmat=f, nomsize=ns, fixed_measured=fm, lmat=lf[:nlm], lmat_of_link=lol[:self.counts()[1]])

    def signals(self):
        """Per voxel: localSignal."""
        out = np.zeros(max(self.counts()[0], 1))
        f = getattr(self.lib, self.p + "signals")
        f.restype, f.argtypes = None, [ctypes.c_void_p, ctypes.c_void_p]
        f(self.h, _P(out))
        return out[:self.counts()[0]]

    def link_offsets(self):
        """Per link: the plastic strain offset of a non-linear material (0 otherwise)."""
        off = np.zeros(max(self.counts()[1], 1), np.float32)
        self._f("link_offsets")(self.h, _P(off))
        return off[:self.counts()[1]]

    def link_curves(self):
        """Per link material: its stress-strain points as an (n, 2) float32 array."""
        out = []
        for i in range(self._f("num_link_mats")(self.h)):
            e, s = np.zeros(128, np.float32), np.zeros(128, np.float32)
            n = self._f("link_curve")(self.h, i, _P(e), _P(s), 128)
            out.append(np.stack([e[:n], s[:n]], 1))
        return out

    def surface(self):
        ns = self.counts()[2]
        idx = np.zeros(max(ns, 1), np.int32)
        self._f("surface")(self.h, _P(idx))
        return idx[:ns]

    def last_contact(self):
        nv = self.counts()[0]
        c = np.zeros((nv, 3))
        self._f("last_contact")(self.h, _P(c))
        return c

    def com(self):
        c = np.zeros(3)
        self._f("com")(self.h, _P(c))
        return c


def robot_struct(robot):
    """Pack a workloads.Robot into the oracle's vxo_robot (lattice with z_offset padding)."""
    g, ph = robot.padded()
    lattice = np.ascontiguousarray(g.reshape(-1).astype(np.uint8))
    phase = None if ph is None else np.ascontiguousarray(ph.reshape(-1).astype(np.float64))
    mats = (VxoMaterial * max(len(robot.materials), 1))()
    ss_keep = []
    for i, m in enumerate(robot.materials):
        n, e, s = m.ss_arrays()
        ss_keep.append((e, s))
        mats[i] = VxoMaterial(m.E, m.nu, m.rho, m.cte, m.mu_static, m.mu_kinetic,
                              m.fail_stress, m.mat_model(), m.fixed, m.is_measured, m.thermal_on_after,
                              m.cilia, m.cilia_on_after, m.remove_after, m.plastic_mod, m.yield_stress,
                              n, None if e is None else _P(e), None if s is None else _P(s),
                              int(m.is_pacemaker), m.pacemaker_period, m.signal_value_decay, m.signal_time_delay,
                              m.inactive_period, int(m.sticky))
    Z, Y, X = g.shape
    r = VxoRobot(X, Y, Z, _P(lattice), None if phase is None else _P(phase), len(robot.materials), mats,
                 robot.vox_size, robot.dt_frac, robot.grav_acc, int(robot.floor),
                 robot.temp_amplitude, robot.temp_period, robot.temp_base, int(robot.temp_enabled), int(robot.temp_vary),
                 int(robot.enable_expansion), int(robot.enable_collision), int(robot.volume_effects),
                 robot.bond_damping, robot.col_damping, robot.slow_damping)
    progs = _force_field_tokens(robot)
    for k, t in enumerate(progs):
        if t is not None:
            r.force_field[k] = _P(t)
    cil = []
    if robot.enable_cilia:
        r.enable_cilia = 1
        for name in ("cilia_base", "cilia_shift"):
            a = robot.padded_cells(getattr(robot, name))
            if a is not None:
                cil.append(a)
                setattr(r, name, _P(a))
    r.enable_detach = int(robot.enable_detach)
    r.secondary_experiment = int(robot.secondary_experiment)
    r.enable_signals = int(robot.enable_signals)
    r.enable_attach = int(robot.enable_attach)
    r.safety_guard = int(robot.safety_guard)
    conds = _attach_tokens(robot)
    for k, t in enumerate(conds):
        if t is not None:
            r.attach_cond[k] = _P(t)
    bcs = None
    if robot.bcs:
        from vx3g.abi import bc_array
        bcs = bc_array(VxoBC, robot.bcs)
        r.n_bcs = len(robot.bcs)
        r.bcs = bcs
    return r, (lattice, phase, mats, progs, cil, ss_keep, bcs, conds)


def _force_field_tokens(robot):
    from vx3g.workloads import math_tokens
    ff = getattr(robot, "force_field", None) or [None] * 3
    return [None if t is None else np.ascontiguousarray(math_tokens(t)) for t in ff]


def _attach_tokens(robot):
    """The five AttachCondition programs (None where absent)."""
    from vx3g.workloads import math_tokens
    conds = list(getattr(robot, "attach_conditions", None) or [])
    conds += [None] * (5 - len(conds))
    return [None if t is None else np.ascontiguousarray(math_tokens(t)) for t in conds[:5]]


def oracle_sim(robot) -> Sim:
    lib = _setup(ctypes.CDLL(build_oracle()), "vxo_")
    lib.vxo_create.restype = ctypes.c_void_p
    lib.vxo_create.argtypes = [ctypes.POINTER(VxoRobot)]
    r, keep = robot_struct(robot)
    h = lib.vxo_create(ctypes.byref(r))
    return Sim(lib, "vxo_", h, (r, keep))


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_sim(robot) -> Sim:
    from vx3g.workloads import to_vxa
    lib = _setup(ctypes.CDLL(REF_SO), "vx3ref_")
    lib.vx3ref_create.restype = ctypes.c_void_p
    lib.vx3ref_create.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    h = lib.vx3ref_create(to_vxa(robot).encode(), int(robot.enable_collision), int(robot.enable_expansion))
    lib.vx3ref_set_force_field.restype = ctypes.c_int
    lib.vx3ref_set_force_field.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    progs = _force_field_tokens(robot)
    for k, t in enumerate(progs):
        if t is not None:
            assert lib.vx3ref_set_force_field(h, k, _P(t), len(t)) == 0
    lib.vx3ref_set_cilia.restype = None
    lib.vx3ref_set_cilia.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.vx3ref_set_cilia(h, int(robot.enable_cilia))
    lib.vx3ref_set_detach.restype = None
    lib.vx3ref_set_detach.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.vx3ref_set_detach(h, int(robot.enable_detach))
    lib.vx3ref_set_secondary.restype = None
    lib.vx3ref_set_secondary.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.vx3ref_set_secondary(h, int(robot.secondary_experiment))
    lib.vx3ref_set_signals.restype = None
    lib.vx3ref_set_signals.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.vx3ref_set_signals(h, int(robot.enable_signals))
    lib.vx3ref_set_attach.restype = None
    lib.vx3ref_set_attach.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.vx3ref_set_attach(h, int(robot.enable_attach), int(robot.safety_guard))
    lib.vx3ref_set_attach_condition.restype = ctypes.c_int
    lib.vx3ref_set_attach_condition.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
    conds = _attach_tokens(robot)
    for k, t in enumerate(conds):
        if t is not None:
            assert lib.vx3ref_set_attach_condition(h, k, _P(t), len(t)) == 0
    return Sim(lib, "vx3ref_", h, (progs, conds))
