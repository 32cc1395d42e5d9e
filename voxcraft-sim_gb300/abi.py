"""ctypes binding of libvx3g.so (include/vx3g.h) and a small batch wrapper.

This is the Python face of the C ABI, used by the tests, the benchmark and the
smoke check.  There is no fallback: if the CUDA library is missing or fails to
load, every entry point raises.
"""

from __future__ import annotations

import ctypes
import os
from typing import List, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libvx3g.so")

PRECISION_FP64 = 0
PRECISION_MIXED = 1
ROBOT_OK, ROBOT_DIVERGED, ROBOT_CONTACT_OVERFLOW, ROBOT_STOPPED = 0, 1, 2, 4

EXPORTS = [
    "vx3g_create", "vx3g_destroy", "vx3g_last_error", "vx3g_step", "vx3g_synchronize", "vx3g_stream",
    "vx3g_counts", "vx3g_offsets", "vx3g_get_state", "vx3g_set_state", "vx3g_get_voxel_aux", "vx3g_get_links",
    "vx3g_get_topology", "vx3g_get_surface", "vx3g_com", "vx3g_dt", "vx3g_time", "vx3g_status",
    "vx3g_steps_taken", "vx3g_time_steps", "vx3g_flush_l2", "vx3g_time_passes", "vx3g_stop_robot",
    "vx3g_record", "vx3g_backward", "vx3g_recommended_dt_noalloc", "vx3g_autotune", "vx3g_launch_shapes",
    "vx3g_debug_barrier", "vx3g_prepare_graphs", "vx3g_get_signals",
]


class Material(ctypes.Structure):
    _fields_ = [("E", ctypes.c_double), ("nu", ctypes.c_double), ("rho", ctypes.c_double), ("cte", ctypes.c_double),
                ("mu_static", ctypes.c_double), ("mu_kinetic", ctypes.c_double), ("fail_stress", ctypes.c_double),
                ("model", ctypes.c_int), ("fixed", ctypes.c_int), ("is_measured", ctypes.c_int),
                ("thermal_on_after", ctypes.c_double), ("cilia", ctypes.c_double), ("cilia_on_after", ctypes.c_double),
                ("remove_after", ctypes.c_double), ("plastic_mod", ctypes.c_double), ("yield_stress", ctypes.c_double),
                ("n_data", ctypes.c_int), ("strain_data", ctypes.c_void_p), ("stress_data", ctypes.c_void_p),
                ("is_pacemaker", ctypes.c_int), ("pacemaker_period", ctypes.c_double),
                ("signal_value_decay", ctypes.c_double), ("signal_time_delay", ctypes.c_double),
                ("inactive_period", ctypes.c_double), ("sticky", ctypes.c_int)]


class BCRegion(ctypes.Structure):
    _fields_ = [("prim", ctypes.c_int), ("dof_fixed", ctypes.c_int), ("x", ctypes.c_float), ("y", ctypes.c_float),
                ("z", ctypes.c_float), ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
                ("radius", ctypes.c_float), ("force", ctypes.c_double * 3), ("torque", ctypes.c_double * 3),
                ("displace", ctypes.c_double * 3), ("ang_displace", ctypes.c_double * 3)]


def bc_array(cls, bcs):
    """ctypes array of `cls` (BCRegion or the oracle's struct of the same layout) from workloads.BCRegion."""
    arr = (cls * max(len(bcs), 1))()
    for i, b in enumerate(bcs):
        arr[i] = cls(int(b.prim), int(b.dof_fixed), b.x, b.y, b.z, b.dx, b.dy, b.dz, b.radius,
                     (ctypes.c_double * 3)(*b.force), (ctypes.c_double * 3)(*b.torque),
                     (ctypes.c_double * 3)(*b.displace), (ctypes.c_double * 3)(*b.ang_displace))
    return arr


class RobotDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("lattice", ctypes.c_void_p), ("phase", ctypes.c_void_p),
                ("n_materials", ctypes.c_int), ("materials", ctypes.POINTER(Material)),
                ("vox_size", ctypes.c_double), ("dt_frac", ctypes.c_double), ("grav_acc", ctypes.c_double),
                ("floor_enabled", ctypes.c_int),
                ("temp_amplitude", ctypes.c_double), ("temp_period", ctypes.c_double), ("temp_base", ctypes.c_double),
                ("temp_enabled", ctypes.c_int), ("vary_temp", ctypes.c_int), ("enable_expansion", ctypes.c_int),
                ("enable_collision", ctypes.c_int), ("volume_effects", ctypes.c_int),
                ("bond_damping", ctypes.c_double), ("col_damping", ctypes.c_double), ("slow_damping", ctypes.c_double),
                ("log10E", ctypes.c_void_p), ("force_field", ctypes.c_void_p * 3),
                ("enable_cilia", ctypes.c_int), ("cilia_base", ctypes.c_void_p), ("cilia_shift", ctypes.c_void_p),
                ("enable_detach", ctypes.c_int), ("secondary_experiment", ctypes.c_int),
                ("n_bcs", ctypes.c_int), ("bcs", ctypes.POINTER(BCRegion)), ("enable_signals", ctypes.c_int),
                ("enable_attach", ctypes.c_int), ("safety_guard", ctypes.c_int),
                ("attach_condition", ctypes.c_void_p * 5)]


class BatchDesc(ctypes.Structure):
    _fields_ = [("n_robots", ctypes.c_int), ("robots", ctypes.POINTER(RobotDesc)), ("precision", ctypes.c_int),
                ("device", ctypes.c_int), ("graph_chunk", ctypes.c_int)]


_lib = None


def load(path: str = LIB_PATH):
    """Load libvx3g.so and declare its signatures (raises if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libvx3g.so not built ({path}); run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p
    lib.vx3g_create.restype = vp
    lib.vx3g_create.argtypes = [ctypes.POINTER(BatchDesc), ctypes.POINTER(ctypes.c_int)]
    lib.vx3g_destroy.restype = None
    lib.vx3g_destroy.argtypes = [vp]
    lib.vx3g_last_error.restype = ctypes.c_char_p
    lib.vx3g_last_error.argtypes = []
    lib.vx3g_step.argtypes = [vp, ip]
    lib.vx3g_synchronize.argtypes = [vp]
    lib.vx3g_stream.restype = vp
    lib.vx3g_stream.argtypes = [vp]
    lib.vx3g_counts.argtypes = [vp, dp, dp, dp]
    lib.vx3g_offsets.argtypes = [vp, dp, dp]
    lib.vx3g_get_state.argtypes = [vp, dp, dp, dp, dp]
    lib.vx3g_set_state.argtypes = [vp, dp, dp, dp, dp]
    lib.vx3g_get_voxel_aux.argtypes = [vp, dp, dp, dp]
    lib.vx3g_get_links.argtypes = [vp, dp, dp, dp, dp, dp]
    lib.vx3g_get_topology.argtypes = [vp, dp, dp, dp, dp]
    lib.vx3g_get_surface.argtypes = [vp, dp]
    for f in ("vx3g_com", "vx3g_dt", "vx3g_time", "vx3g_status"):
        getattr(lib, f).argtypes = [vp, dp]
    lib.vx3g_steps_taken.restype = ctypes.c_int64
    lib.vx3g_steps_taken.argtypes = [vp]
    lib.vx3g_time_steps.argtypes = [vp, ip, dp]
    lib.vx3g_flush_l2.argtypes = [vp, ctypes.c_size_t]
    lib.vx3g_time_passes.argtypes = [vp, ip, dp]
    lib.vx3g_stop_robot.argtypes = [vp, ip]
    lib.vx3g_record.argtypes = [vp, ip, ip]
    lib.vx3g_recommended_dt_noalloc.argtypes = [vp, dp]
    lib.vx3g_autotune.argtypes = [vp, ip, ctypes.c_char_p]
    lib.vx3g_launch_shapes.argtypes = [vp, vp]
    lib.vx3g_backward.argtypes = [vp, dp, dp, dp]
    lib.vx3g_debug_barrier.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32]
    lib.vx3g_prepare_graphs.argtypes = [vp]
    lib.vx3g_get_signals.argtypes = [vp, dp]
    lib.vx3g_links_in_use.argtypes = [vp, dp]
    _lib = lib
    return lib


def _P(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Vx3gError(RuntimeError):
    pass


def _check(rc, what):
    if rc != 0:
        raise Vx3gError(f"{what} failed ({rc}): {_lib.vx3g_last_error().decode()}")


def robot_desc(robot):
    """Pack a workloads.Robot into a RobotDesc; returns (desc, keep-alive objects)."""
    g, ph = robot.padded()
    lattice = np.ascontiguousarray(g.reshape(-1).astype(np.uint8))
    phase = None if ph is None else np.ascontiguousarray(ph.reshape(-1).astype(np.float64))
    mats = (Material * len(robot.materials))()
    ss_keep = []
    for i, m in enumerate(robot.materials):
        n, e, s = m.ss_arrays()
        ss_keep.append((e, s))
        mats[i] = Material(m.E, m.nu, m.rho, m.cte, m.mu_static, m.mu_kinetic, m.fail_stress,
                           m.mat_model(), int(m.fixed), int(m.is_measured), float(m.thermal_on_after),
                           float(m.cilia), float(m.cilia_on_after), float(m.remove_after),
                           float(m.plastic_mod), float(m.yield_stress), n, _P(e), _P(s),
                           int(m.is_pacemaker), float(m.pacemaker_period), float(m.signal_value_decay),
                           float(m.signal_time_delay), float(m.inactive_period), int(m.sticky))
    Z, Y, X = g.shape
    log10E = getattr(robot, "log10E", None)
    if log10E is not None:
        le = log10E
        if robot.z_offset:
            le = np.concatenate([np.zeros((robot.z_offset,) + le.shape[1:]), le], axis=0)
        log10E = np.ascontiguousarray(le.reshape(-1).astype(np.float64))
    d = RobotDesc(X, Y, Z, _P(lattice), _P(phase), len(robot.materials), mats, robot.vox_size, robot.dt_frac,
                  robot.grav_acc, int(robot.floor), robot.temp_amplitude, robot.temp_period, robot.temp_base,
                  int(robot.temp_enabled),
                  int(robot.temp_vary), int(robot.enable_expansion), int(robot.enable_collision),
                  int(robot.volume_effects), robot.bond_damping, robot.col_damping, robot.slow_damping,
                  _P(log10E))
    from . import workloads as wl  # noqa: E402  (math-tree token layout)
    progs = []
    for k, tree in enumerate(getattr(robot, "force_field", None) or [None] * 3):
        if tree is not None:
            progs.append(np.ascontiguousarray(wl.math_tokens(tree)))
            d.force_field[k] = _P(progs[-1])
    d.enable_detach = int(robot.enable_detach)
    d.secondary_experiment = int(robot.secondary_experiment)
    cil = []
    if robot.enable_cilia:
        d.enable_cilia = 1
        for name in ("cilia_base", "cilia_shift"):
            a = robot.padded_cells(getattr(robot, name))
            if a is not None:
                cil.append(a)
                setattr(d, name, _P(a))
    d.enable_signals = int(robot.enable_signals)
    d.enable_attach = int(robot.enable_attach)
    d.safety_guard = int(robot.safety_guard)
    for k, tree in enumerate((getattr(robot, "attach_conditions", None) or [])[:5]):
        if tree is not None:
            progs.append(np.ascontiguousarray(wl.math_tokens(tree)))
            d.attach_condition[k] = _P(progs[-1])
    bcs = None
    if robot.bcs:
        bcs = bc_array(BCRegion, robot.bcs)
        d.n_bcs = len(robot.bcs)
        d.bcs = bcs
    return d, (lattice, phase, mats, log10E, progs, cil, ss_keep, bcs)


class Batch:
    """A vx3g context holding a batch of robots on one GPU."""

    def __init__(self, robots: Sequence, precision: int = PRECISION_FP64, device: int = 0, graph_chunk: int = 100):
        lib = load()
        self.lib = lib
        descs = (RobotDesc * len(robots))()
        self._keep = []
        for i, r in enumerate(robots):
            d, keep = robot_desc(r)
            descs[i] = d
            self._keep.append(keep)
        bd = BatchDesc(len(robots), descs, precision, device, graph_chunk)
        st = ctypes.c_int(0)
        h = lib.vx3g_create(ctypes.byref(bd), ctypes.byref(st))
        if not h:
            raise Vx3gError(f"vx3g_create failed ({st.value}): {lib.vx3g_last_error().decode()}")
        self.h = ctypes.c_void_p(h)
        self.n_robots = len(robots)
        nv, nl, ns = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib.vx3g_counts(self.h, ctypes.byref(nv), ctypes.byref(nl), ctypes.byref(ns)), "vx3g_counts")
        self.nv, self.nl, self.ns = nv.value, nl.value, ns.value
        vo = np.zeros(self.n_robots + 1, np.int32)
        lo = np.zeros(self.n_robots + 1, np.int32)
        _check(lib.vx3g_offsets(self.h, _P(vo), _P(lo)), "vx3g_offsets")
        self.voxel_offset, self.link_offset = vo, lo

    def close(self):
        if getattr(self, "h", None):
            self.lib.vx3g_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n: int):
        _check(self.lib.vx3g_step(self.h, int(n)), "vx3g_step")

    def prepare_graphs(self):
        """Capture the step graphs now (vx3g_prepare_graphs), outside any timed region."""
        _check(self.lib.vx3g_prepare_graphs(self.h), "vx3g_prepare_graphs")

    def synchronize(self):
        _check(self.lib.vx3g_synchronize(self.h), "vx3g_synchronize")

    def stream(self) -> int:
        return self.lib.vx3g_stream(self.h)

    def steps_taken(self) -> int:
        return self.lib.vx3g_steps_taken(self.h)

    def state(self, out=None):
        """Voxel state as float64 arrays; `out` (a dict of C-contiguous float64 arrays
        with the keys and shapes returned here) is filled in place instead."""
        if out is None:
            pos, lm, am = (np.zeros((self.nv, 3)) for _ in range(3))
            orient = np.zeros((self.nv, 4))
            out = dict(pos=pos, orient=orient, linmom=lm, angmom=am)
        for k, comps in (("pos", 3), ("orient", 4), ("linmom", 3), ("angmom", 3)):
            a = out[k]
            if a.dtype != np.float64 or a.shape != (self.nv, comps) or not a.flags.c_contiguous:
                raise ValueError(f"state(out=...): {k} must be a C-contiguous float64 array of shape ({self.nv}, {comps})")
        _check(self.lib.vx3g_get_state(self.h, _P(out["pos"]), _P(out["orient"]), _P(out["linmom"]),
                                       _P(out["angmom"])), "vx3g_get_state")
        return out

    def set_state(self, pos=None, orient=None, linmom=None, angmom=None):
        c = lambda a: None if a is None else np.ascontiguousarray(a, np.float64)
        pos, orient, linmom, angmom = c(pos), c(orient), c(linmom), c(angmom)
        _check(self.lib.vx3g_set_state(self.h, _P(pos), _P(orient), _P(linmom), _P(angmom)), "vx3g_set_state")

    def voxel_aux(self):
        tempe = np.zeros(self.nv, np.float32)
        flags = np.zeros(self.nv, np.int32)
        contact = np.zeros((self.nv, 3))
        _check(self.lib.vx3g_get_voxel_aux(self.h, _P(tempe), _P(flags), _P(contact)), "vx3g_get_voxel_aux")
        return dict(tempe=tempe, flags=flags, contact=contact)

    def links(self):
        strain, maxs = np.zeros(self.nl, np.float32), np.zeros(self.nl, np.float32)
        local9, forces = np.zeros((self.nl, 9)), np.zeros((self.nl, 12))
        small = np.zeros(self.nl, np.int32)
        _check(self.lib.vx3g_get_links(self.h, _P(strain), _P(maxs), _P(local9), _P(forces), _P(small)),
               "vx3g_get_links")
        return dict(strain=strain, maxstrain=maxs, local9=local9, forces=forces, small=small)

    def links_in_use(self):
        """Per robot: its lattice's links plus those attachment has made (the first entries
        of its link range; the rest of the range is unused reserve)."""
        out = np.zeros(self.n_robots, np.int32)
        _check(self.lib.vx3g_links_in_use(self.h, _P(out)), "vx3g_links_in_use")
        return out

    def signals(self):
        """Per voxel: localSignal (0 in robots without signals)."""
        out = np.zeros(self.nv)
        _check(self.lib.vx3g_get_signals(self.h, _P(out)), "vx3g_get_signals")
        return out

    def topology(self):
        ijk = np.zeros((self.nv, 3), np.int32)
        mat = np.zeros(self.nv, np.int32)
        ends = np.zeros((self.nl, 2), np.int32)
        axis = np.zeros(self.nl, np.int32)
        _check(self.lib.vx3g_get_topology(self.h, _P(ijk), _P(mat), _P(ends), _P(axis)), "vx3g_get_topology")
        return dict(ijk=ijk, mat=mat, negpos=ends, axis=axis)

    def surface(self):
        """Surface voxels (fewer than six links) now; the set grows when links detach."""
        nv, nl, ns = (ctypes.c_int(), ctypes.c_int(), ctypes.c_int())
        _check(self.lib.vx3g_counts(self.h, ctypes.byref(nv), ctypes.byref(nl), ctypes.byref(ns)), "vx3g_counts")
        s = np.zeros(max(ns.value, 1), np.int32)
        _check(self.lib.vx3g_get_surface(self.h, _P(s)), "vx3g_get_surface")
        return s[:ns.value]

    def com(self):
        c = np.zeros((self.n_robots, 3))
        _check(self.lib.vx3g_com(self.h, _P(c)), "vx3g_com")
        return c

    def dt(self):
        d = np.zeros(self.n_robots)
        _check(self.lib.vx3g_dt(self.h, _P(d)), "vx3g_dt")
        return d

    def time(self):
        t = np.zeros(self.n_robots)
        _check(self.lib.vx3g_time(self.h, _P(t)), "vx3g_time")
        return t

    def time_steps(self, n: int) -> float:
        """Device milliseconds for vx3g_step(n), timed with CUDA events on the context stream."""
        ms = np.zeros(1, np.float32)
        _check(self.lib.vx3g_time_steps(self.h, int(n), _P(ms)), "vx3g_time_steps")
        return float(ms[0])

    def flush_l2(self, nbytes: int = 512 << 20):
        _check(self.lib.vx3g_flush_l2(self.h, int(nbytes)), "vx3g_flush_l2")

    def time_passes(self, iters: int = 50):
        ms = np.zeros(4, np.float32)
        _check(self.lib.vx3g_time_passes(self.h, int(iters), _P(ms)), "vx3g_time_passes")
        return dict(links=float(ms[0]), collision=float(ms[1]), voxels=float(ms[2]), contact_eval=float(ms[3]))

    def record(self, n: int, checkpoint_every: int = 100):
        _check(self.lib.vx3g_record(self.h, int(n), int(checkpoint_every)), "vx3g_record")

    def backward(self, dL_dcom):
        w = np.ascontiguousarray(np.asarray(dL_dcom, np.float64).reshape(self.n_robots, 3))
        gp = np.zeros(self.nv)
        ge = np.zeros(self.nv)
        _check(self.lib.vx3g_backward(self.h, _P(w), _P(gp), _P(ge)), "vx3g_backward")
        return gp, ge

    def autotune(self, n_steps: int, cache_json=None):
        c = None if cache_json is None else str(cache_json).encode()
        _check(self.lib.vx3g_autotune(self.h, int(n_steps), c), "vx3g_autotune")

    def launch_shapes(self):
        out = np.zeros(4, np.int32)
        _check(self.lib.vx3g_launch_shapes(self.h, _P(out)), "vx3g_launch_shapes")
        return out

    def recommended_dt_noalloc(self):
        out = np.zeros(self.n_robots)
        _check(self.lib.vx3g_recommended_dt_noalloc(self.h, _P(out)), "vx3g_recommended_dt_noalloc")
        return out

    def debug_barrier(self, polls: int, arrivals: int):
        """Test hook: make the next list rebuild's grid barrier give up (vx3g_debug_barrier)."""
        _check(self.lib.vx3g_debug_barrier(self.h, int(polls), int(arrivals)), "vx3g_debug_barrier")

    def stop_robot(self, r: int):
        _check(self.lib.vx3g_stop_robot(self.h, int(r)), "vx3g_stop_robot")

    def status(self):
        s = np.zeros(self.n_robots, np.int32)
        _check(self.lib.vx3g_status(self.h, _P(s)), "vx3g_status")
        return s
