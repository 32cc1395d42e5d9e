"""Seeded synthetic robots in the reference's VXA format.

The reference ships no benchmark suite or dataset; every workload here is
generated from a seed.  A robot is a dense lattice of material ids
(0 = empty, 1..K = palette entry) plus per-voxel actuation phase, written out
as a VXA document that the reference's own reader accepts
(src/VXA/VX_Object.cpp:1760-1884 for <Structure> with ASCII_READABLE layers
and <PhaseOffset> rows; src/VXA/VX_Sim.cpp:185-294 for <Simulator>;
src/old/VX_Environment.cpp:150-172 for <Environment>).

Robot generators follow the workload descriptions:
  * solid_block    -- n x n x n solid cube of one passive material
  * bernoulli_body -- Bernoulli(p) fill, largest 6-connected component kept
"""

from __future__ import annotations

import dataclasses
from collections import deque
from typing import List, Optional, Sequence

import numpy as np


@dataclasses.dataclass
class Material:
    E: float = 1e6
    nu: float = 0.35
    rho: float = 1e3
    cte: float = 0.0
    mu_static: float = 1.0
    mu_kinetic: float = 0.5
    fail_stress: float = 0.0   # 0 -> linear model without failure (MatModel 0)
    fixed: int = 0
    is_measured: int = 1
    cilia: float = 0.0         # Cilia (scale of the cilia force)
    cilia_on_after: float = 0.0  # TurnOnCiliaAfterThisManySeconds
    remove_after: float = 0.0  # RemoveFromSimulationAfterThisManySeconds (SecondaryExperiment; 0: never)
    thermal_on_after: float = 0.0  # TurnOnThermalExpansionAfterThisManySeconds (actuation starts then)
    name: str = "mat"
    model: Optional[int] = None  # MatModel (0 linear, 1 linear+failure, 2 bilinear, 3 data points);
                                 # None: 0 without fail_stress, 1 with
    plastic_mod: float = 0.0   # Plastic_Mod (MatModel 2)
    yield_stress: float = 0.0  # Yield_Stress (MatModel 2)
    ss_strain: Optional[tuple] = None  # SSData strain points (MatModel 3), (0, 0) first as in a VXA
    ss_stress: Optional[tuple] = None  # SSData stress points (MatModel 3)
    is_pacemaker: int = 0              # isPaceMaker: emits a signal every pacemaker_period seconds
    pacemaker_period: float = 0.0      # PaceMakerPeriod
    signal_value_decay: float = 0.9    # signalValueDecay
    signal_time_delay: float = 0.03    # signalTimeDelay
    inactive_period: float = 0.03      # inactivePeriod
    sticky: int = 0                    # Sticky: with EnableAttach, touching voxels of this material link up

    def mat_model(self) -> int:
        if self.model is not None:
            return int(self.model)
        return 0 if self.fail_stress == 0 else 1

    def ss_arrays(self):
        """(n, strain float64 array, stress float64 array) of the SSData points, or (0, None, None)."""
        if self.mat_model() != 3 or self.ss_strain is None:
            return 0, None, None
        e = np.ascontiguousarray(self.ss_strain, np.float64)
        s = np.ascontiguousarray(self.ss_stress, np.float64)
        return len(e), e, s


@dataclasses.dataclass
class BCRegion:
    """An <Environment><Boundary_Conditions> region (FRegion): every voxel it touches has
    the fixed DOFs held at their displacement and a share of the force and torque.
    Coordinates are fractions of the workspace (the lattice's extent)."""
    prim: int = 0              # PrimType: 0 box, 1 cylinder, 2 sphere
    dof_fixed: int = 0         # DofFixed: 1 X, 2 Y, 4 Z translation; 8 X, 16 Y, 32 Z rotation
    x: float = 0.0
    y: float = 0.0
    z: float = 0.0
    dx: float = 0.0
    dy: float = 0.0
    dz: float = 0.0
    radius: float = 0.0
    force: tuple = (0.0, 0.0, 0.0)
    torque: tuple = (0.0, 0.0, 0.0)
    displace: tuple = (0.0, 0.0, 0.0)
    ang_displace: tuple = (0.0, 0.0, 0.0)


@dataclasses.dataclass
class Robot:
    """One simulation: lattice (z, y, x) of palette indices and its settings."""
    grid: np.ndarray                      # int8/uint8 [Z, Y, X], 0 = empty
    materials: List[Material]
    phase: Optional[np.ndarray] = None    # float64 [Z, Y, X] in cycles (only occupied cells read)
    vox_size: float = 0.01
    z_offset: int = 0                     # lattice cells added below the body (drop height)
    dt_frac: float = 0.9
    bond_damping: float = 1.0
    col_damping: float = 1.0
    slow_damping: float = 0.0
    gravity: bool = True
    grav_acc: float = -9.81
    floor: bool = True
    temp_vary: bool = False
    temp_amplitude: float = 0.0
    temp_period: float = 0.2
    temp_base: float = 25.0
    temp_enabled: bool = False            # Environment/Thermal/TempEnabled: without VaryTempEnabled, every voxel
                                          # starts (and stays) at TempBase + TempAmplitude (static expansion)
    enable_expansion: int = 0
    enable_collision: bool = False
    volume_effects: bool = True
    log10E: Optional[np.ndarray] = None   # float64 [Z, Y, X] per-voxel log10 E (C ABI only; not in VXA)
    force_field: Optional[list] = None    # Simulator/ForceField: [x, y, z] math trees (see math_tokens) or None
    enable_cilia: bool = False            # Simulator/EnableCilia
    enable_detach: bool = False           # Simulator/AttachDetach/EnableDetach (failed links leave the lattice)
    secondary_experiment: bool = False    # Simulator/SecondaryExperiment (material removal, initial-position reset)
    reinit_after: float = 0.0             # Simulator/ReinitializeInitialPositionAfterThisManySeconds
    cilia_base: Optional[np.ndarray] = None   # float64 [Z, Y, X, 3] BaseCiliaForce (only occupied cells read)
    cilia_shift: Optional[np.ndarray] = None  # float64 [Z, Y, X, 3] ShiftCiliaForce
    stop_time: Optional[float] = None     # StopConditionFormula "t - stop_time" (> 0 stops)
    stop_formula: Optional[tuple] = None  # or any StopConditionFormula math tree (see math_tokens)
    fitness_x: bool = False               # FitnessFunction "x" (COM displacement along x)
    record_step: int = 0                  # RecordHistory/RecordStepSize
    bcs: Optional[list] = None            # Environment/Boundary_Conditions: BCRegion list
    enable_signals: bool = False          # Simulator/EnableSignals
    enable_attach: bool = False           # Simulator/AttachDetach/EnableAttach (runtime links between Sticky voxels)
    safety_guard: int = 500               # Simulator/AttachDetach/SafetyGuard: a new link's forces are scaled
                                          # by 0.01 for its first this many updates
    attach_conditions: Optional[list] = None  # AttachDetach/AttachCondition/Condition_0..4: up to five math
                                              # trees (None entries absent); a voxel may attach while all > 0

    def occupied(self) -> np.ndarray:
        return self.grid > 0

    def padded_cells(self, a):
        """A per-cell [Z, Y, X, ...] array with the z_offset empty layers below, flattened
        (x fastest), or None."""
        if a is None:
            return None
        if self.z_offset:
            a = np.concatenate([np.zeros((self.z_offset,) + a.shape[1:], a.dtype), a], axis=0)
        return np.ascontiguousarray(a.reshape(-1).astype(np.float64))

    def padded(self):
        """Lattice with z_offset empty layers underneath, as written to the VXA."""
        g = self.grid
        if self.z_offset:
            pad = np.zeros((self.z_offset,) + g.shape[1:], dtype=g.dtype)
            g = np.concatenate([pad, g], axis=0)
        ph = self.phase
        if ph is not None and self.z_offset:
            pad = np.zeros((self.z_offset,) + ph.shape[1:], dtype=ph.dtype)
            ph = np.concatenate([pad, ph], axis=0)
        return g, ph


def largest_component(mask: np.ndarray) -> np.ndarray:
    """Largest 6-connected component of a boolean [Z, Y, X] mask."""
    Z, Y, X = mask.shape
    label = np.zeros(mask.shape, dtype=np.int32)
    best, best_n, cur = 0, 0, 0
    for z, y, x in zip(*np.nonzero(mask)):
        if label[z, y, x]:
            continue
        cur += 1
        n = 0
        q = deque([(z, y, x)])
        label[z, y, x] = cur
        while q:
            a, b, c = q.popleft()
            n += 1
            for da, db, dc in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
                na, nb, nc = a + da, b + db, c + dc
                if 0 <= na < Z and 0 <= nb < Y and 0 <= nc < X and mask[na, nb, nc] and not label[na, nb, nc]:
                    label[na, nb, nc] = cur
                    q.append((na, nb, nc))
        if n > best_n:
            best, best_n = cur, n
    return label == best if best else np.zeros_like(mask)


def solid_block(n: int = 10, drop_cells: int = 2, material: Optional[Material] = None, **kw) -> Robot:
    """n^3 solid block of one material, dropped from drop_cells lattice units."""
    m = material or Material(E=1e6, nu=0.35, rho=1e3, cte=0.0, mu_static=1.0, mu_kinetic=0.5)
    grid = np.ones((n, n, n), dtype=np.uint8)
    return Robot(grid=grid, materials=[m], z_offset=drop_cells, **kw)


def bernoulli_body(rng: np.random.Generator, dims: Sequence[int], p: float, materials: List[Material],
                   random_phase: bool = False, **kw) -> Robot:
    """Bernoulli(p) fill of a dims=(X, Y, Z) box, largest 6-connected component,
    materials drawn uniformly per voxel, optional uniform phase in cycles [0,1)."""
    X, Y, Z = dims
    mask = rng.random((Z, Y, X)) < p
    mask = largest_component(mask)
    mats = rng.integers(1, len(materials) + 1, size=(Z, Y, X)).astype(np.uint8)
    grid = np.where(mask, mats, 0).astype(np.uint8)
    phase = None
    if random_phase:
        # phase offsets in cycles; 2*pi*phase is the phase angle in [0, 2*pi)
        phase = rng.random((Z, Y, X))
    return Robot(grid=grid, materials=materials, phase=phase, **kw)


# ------------------------------------------------------------------ math trees
# A math tree is a nested tuple (op, arg...): ("mtCONST", 1.5), ("mtVAR", "z"),
# ("mtSUB", a, b) = a - b.  Operator codes are VX3_MathTreeOperator's order
# (src/Utils/VX3_MathTree.h:4-28); variables are the mtVAR names of
# VX3_SimulationManager::ParseMathTree (src/VX3/VX3_SimulationManager.cu:193-217).
MT_OPS = ["mtEND", "mtCONST", "mtE", "mtPI", "mtVAR", "mtADD", "mtSUB", "mtMUL", "mtDIV", "mtPOW", "mtSQRT", "mtSIN",
          "mtCOS", "mtTAN", "mtATAN", "mtLOG", "mtINT", "mtABS", "mtNOT", "mtGREATERTHAN", "mtLESSTHAN", "mtAND",
          "mtOR", "mtNORMALCDF"]
MT_VARS = ["x", "y", "z", "hit", "t", "angle", "targetCloseness", "numClosePairs", "num_voxel"]


def math_tokens(tree) -> np.ndarray:
    """(op, value) tokens of a math tree in the order ParseMathTree writes them
    (src/VX3/VX3_SimulationManager.cu:157-275): every element below the formula
    element, breadth first in document order, pushed on a stack after mtEND and
    popped back, so the program runs leaves-first and ends with mtEND."""
    order = []
    frontier = [tree]
    order.append(tree)
    while frontier:
        nxt = []
        for node in frontier:
            for child in node[1:]:
                if isinstance(child, tuple):
                    order.append(child)
                    nxt.append(child)
        frontier = nxt
    toks = []
    for node in reversed(order):
        op = node[0]
        if op == "mtCONST":
            toks.append((1, 0, float(node[1])))
        elif op == "mtVAR":
            toks.append((4, 0, float(MT_VARS.index(node[1]))))
        else:
            toks.append((MT_OPS.index(op), 0, 0.0))
    toks.append((0, 0, 0.0))
    return np.array(toks, dtype=[("op", np.int32), ("reserved", np.int32), ("value", np.float64)])


def math_tree_xml(tree) -> str:
    op = tree[0]
    if op == "mtCONST":
        return f"<mtCONST>{_fmt(tree[1])}</mtCONST>"
    if op == "mtVAR":
        return f"<mtVAR>{tree[1]}</mtVAR>"
    return f"<{op}>" + "".join(math_tree_xml(c) for c in tree[1:]) + f"</{op}>"


def _fmt(v: float) -> str:
    return repr(float(v))


def structure_xml(r: Robot, replace: Optional[str] = None) -> str:
    """The <Structure> element (ASCII_READABLE layers, optional PhaseOffset rows);
    with replace="VXA.VXC.Structure" it is a VXD override of a base VXA."""
    g, ph = r.padded()
    Z, Y, X = g.shape
    attr = f' replace="{replace}"' if replace else ""
    out = [f'<Structure{attr} Compression="ASCII_READABLE">',
           f"<X_Voxels>{X}</X_Voxels><Y_Voxels>{Y}</Y_Voxels><Z_Voxels>{Z}</Z_Voxels>", "<Data>"]
    for z in range(Z):
        out.append("<Layer><![CDATA[" + "".join(str(int(v)) for v in g[z].reshape(-1)) + "]]></Layer>")
    out.append("</Data>")
    if ph is not None:
        out.append("<PhaseOffset>")
        for z in range(Z):
            out.append("<Layer><![CDATA[" + ",".join(repr(float(v)) for v in ph[z].reshape(-1)) + "]]></Layer>")
        out.append("</PhaseOffset>")
    for tag, a in (("BaseCiliaForce", r.cilia_base), ("ShiftCiliaForce", r.cilia_shift)):
        if a is None:
            continue
        cells = r.padded_cells(a).reshape(Z, Y * X * 3)
        out.append(f"<{tag}>")
        for z in range(Z):
            out.append("<Layer><![CDATA[" + ",".join(repr(float(v)) for v in cells[z]) + "]]></Layer>")
        out.append(f"</{tag}>")
    out.append("</Structure>")
    return "\n".join(out)


def to_vxd(r: Robot) -> str:
    """A VXD document that replaces the base VXA's structure with this robot's."""
    return "<VXD>\n" + structure_xml(r, replace="VXA.VXC.Structure") + "\n</VXD>\n"


def _ss_xml(m: Material) -> str:
    """<SSData> of a MatModel 3 material (src/VXA/VX_Object.cpp:1397-1418)."""
    n, e, s = m.ss_arrays()
    if not n:
        return ""
    return (f"<SSData><NumDataPts>{n}</NumDataPts><StrainData>" + "".join(f"<Strain>{_fmt(x)}</Strain>" for x in e)
            + "</StrainData><StressData>" + "".join(f"<Stress>{_fmt(x)}</Stress>" for x in s)
            + "</StressData></SSData>")


def _bcs_xml(r: Robot) -> str:
    """<Boundary_Conditions> (src/old/VX_Environment.cpp:101-117, VX_FRegion.cpp:165-219)."""
    if not r.bcs:
        return ""
    out = [f"<Boundary_Conditions><NumBCs>{len(r.bcs)}</NumBCs>"]
    for b in r.bcs:
        vals = [("PrimType", b.prim), ("X", b.x), ("Y", b.y), ("Z", b.z), ("dX", b.dx), ("dY", b.dy), ("dZ", b.dz),
                ("Radius", b.radius), ("DofFixed", b.dof_fixed)]
        vals += [(f"Force{a}", v) for a, v in zip("XYZ", b.force)] + [(f"Torque{a}", v) for a, v in zip("XYZ", b.torque)]
        vals += [(f"Displace{a}", v) for a, v in zip("XYZ", b.displace)]
        vals += [(f"AngDisplace{a}", v) for a, v in zip("XYZ", b.ang_displace)]
        out.append("<FRegion>" + "".join(f"<{k}>{_fmt(v) if isinstance(v, float) else v}</{k}>" for k, v in vals)
                   + "</FRegion>")
    out.append("</Boundary_Conditions>")
    return "".join(out)


def to_vxa(r: Robot) -> str:
    """Serialise a Robot as a self-contained VXA document."""
    g, ph = r.padded()
    Z, Y, X = g.shape
    if len(r.materials) > 9:
        raise ValueError("ASCII_READABLE layers hold palette indices 0..9")
    out = ['<VXA Version="1.1">', "<Simulator>",
           f"<Integration><DtFrac>{_fmt(r.dt_frac)}</DtFrac></Integration>",
           "<Damping>"
           f"<BondDampingZ>{_fmt(r.bond_damping)}</BondDampingZ>"
           f"<ColDampingZ>{_fmt(r.col_damping)}</ColDampingZ>"
           f"<SlowDampingZ>{_fmt(r.slow_damping)}</SlowDampingZ>"
           "</Damping>",
           f"<Features><VolumeEffectsEnabled>{int(r.volume_effects)}</VolumeEffectsEnabled></Features>",
           f"<AttachDetach><EnableCollision>{int(r.enable_collision)}</EnableCollision>"
           f"<EnableAttach>{int(r.enable_attach)}</EnableAttach><EnableDetach>{int(r.enable_detach)}</EnableDetach>"
           + (f"<SafetyGuard>{int(r.safety_guard)}</SafetyGuard>" if r.enable_attach else "")
           + ("<AttachCondition>" + "".join(f"<Condition_{i}>{math_tree_xml(t)}</Condition_{i}>"
                                            for i, t in enumerate(r.attach_conditions) if t is not None)
              + "</AttachCondition>" if r.enable_attach and r.attach_conditions else "")
           + "</AttachDetach>",
           f"<EnableExpansion>{int(r.enable_expansion)}</EnableExpansion>",
           *([f"<EnableCilia>1</EnableCilia>"] if r.enable_cilia else []),
           *([f"<EnableSignals>1</EnableSignals>"] if r.enable_signals else []),
           *([f"<SecondaryExperiment>1</SecondaryExperiment><ReinitializeInitialPositionAfterThisManySeconds>"
              f"{_fmt(r.reinit_after)}</ReinitializeInitialPositionAfterThisManySeconds>"]
             if r.secondary_experiment else []),
           *([f"<StopCondition><StopConditionFormula><mtSUB><mtVAR>t</mtVAR><mtCONST>{_fmt(r.stop_time)}</mtCONST>"
              "</mtSUB></StopConditionFormula></StopCondition>"] if r.stop_time is not None else []),
           *([f"<StopCondition><StopConditionFormula>{math_tree_xml(r.stop_formula)}</StopConditionFormula>"
              "</StopCondition>"] if r.stop_formula is not None and r.stop_time is None else []),
           *(["<FitnessFunction><mtVAR>x</mtVAR></FitnessFunction>"] if r.fitness_x else []),
           *(["<ForceField>" + "".join(f"<{a}_forcefield>{math_tree_xml(t)}</{a}_forcefield>"
                                        for a, t in zip("xyz", r.force_field) if t is not None) + "</ForceField>"]
             if r.force_field else []),
           *([f"<RecordHistory><RecordStepSize>{int(r.record_step)}</RecordStepSize><RecordVoxel>1</RecordVoxel>"
              "<RecordLink>0</RecordLink></RecordHistory>"] if r.record_step else []),
           "</Simulator>",
           "<Environment>",
           _bcs_xml(r),
           f"<Gravity><GravEnabled>{int(r.gravity)}</GravEnabled><GravAcc>{_fmt(r.grav_acc)}</GravAcc>"
           f"<FloorEnabled>{int(r.floor)}</FloorEnabled></Gravity>",
           f"<Thermal><TempEnabled>{int(r.temp_enabled)}</TempEnabled>"
           f"<TempAmplitude>{_fmt(r.temp_amplitude)}</TempAmplitude><TempBase>{_fmt(r.temp_base)}</TempBase>"
           f"<VaryTempEnabled>{int(r.temp_vary)}</VaryTempEnabled><TempPeriod>{_fmt(r.temp_period)}</TempPeriod>"
           "</Thermal>",
           "</Environment>",
           '<VXC Version="0.94">',
           f"<Lattice><Lattice_Dim>{_fmt(r.vox_size)}</Lattice_Dim></Lattice>",
           "<Palette>"]
    for i, m in enumerate(r.materials):
        out.append(
            f'<Material ID="{i + 1}"><Name>{m.name}{i + 1}</Name>'
            "<Display><Red>0.5</Red><Green>0.5</Green><Blue>0.5</Blue><Alpha>1</Alpha></Display>"
            "<Mechanical>"
            f"<MatModel>{m.mat_model()}</MatModel>"
            + _ss_xml(m) +
            f"<Elastic_Mod>{_fmt(m.E)}</Elastic_Mod><Fail_Stress>{_fmt(m.fail_stress)}</Fail_Stress>"
            f"<Plastic_Mod>{_fmt(m.plastic_mod)}</Plastic_Mod><Yield_Stress>{_fmt(m.yield_stress)}</Yield_Stress>"
            f"<Density>{_fmt(m.rho)}</Density><Poissons_Ratio>{_fmt(m.nu)}</Poissons_Ratio>"
            f"<CTE>{_fmt(m.cte)}</CTE><MaterialTempPhase>0</MaterialTempPhase>"
            f"<Cilia>{_fmt(m.cilia)}</Cilia><TurnOnCiliaAfterThisManySeconds>{_fmt(m.cilia_on_after)}"
            "</TurnOnCiliaAfterThisManySeconds>"
            f"<RemoveFromSimulationAfterThisManySeconds>{_fmt(m.remove_after)}</RemoveFromSimulationAfterThisManySeconds>"
            f"<TurnOnThermalExpansionAfterThisManySeconds>{_fmt(m.thermal_on_after)}"
            "</TurnOnThermalExpansionAfterThisManySeconds>"
            f"<uStatic>{_fmt(m.mu_static)}</uStatic><uDynamic>{_fmt(m.mu_kinetic)}</uDynamic>"
            f"<Fixed>{int(m.fixed)}</Fixed><Sticky>{int(m.sticky)}</Sticky><isMeasured>{int(m.is_measured)}</isMeasured>"
            f"<isPaceMaker>{int(m.is_pacemaker)}</isPaceMaker><PaceMakerPeriod>{_fmt(m.pacemaker_period)}</PaceMakerPeriod>"
            f"<signalValueDecay>{_fmt(m.signal_value_decay)}</signalValueDecay>"
            f"<signalTimeDelay>{_fmt(m.signal_time_delay)}</signalTimeDelay>"
            f"<inactivePeriod>{_fmt(m.inactive_period)}</inactivePeriod>"
            "</Mechanical></Material>")
    out.append("</Palette>")
    out.append(structure_xml(r))
    out.append("</VXC>")
    out.append("</VXA>")
    return "\n".join(out)


# ------------------------------------------------------------------ sharding
def shard(n_robots: int, rank: int, world: int):
    """The contiguous robot range [lo, hi) that rank `rank` of `world` simulates when a
    population is split across GPUs: robots are independent (no inter-robot forces), so
    each rank steps its range as a batch of its own and no data crosses ranks.  The
    ranges cover 0..n_robots-1 exactly once, in order, sizes differing by at most one."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    base, extra = divmod(n_robots, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


# ------------------------------------------------------------------ named workloads
def c1_block_drop() -> List[Robot]:
    """Plain FP64 reference method: 10x10x10 solid block (E=1e6 Pa, Poisson 0.35,
    1e3 kg/m^3, 0.01 m voxels, bond damping 1.0) dropped from 0.02 m onto a
    floor with mu_s=1, mu_k=0.5; gravity on, collisions off."""
    m = Material(E=1e6, nu=0.35, rho=1e3, mu_static=1.0, mu_kinetic=0.5)
    return [solid_block(10, drop_cells=2, material=m, bond_damping=1.0, col_damping=1.0, slow_damping=0.0)]


def c2_single_body(seed: int = 0, n: int = 64) -> List[Robot]:
    """Single large body: n^3 Bernoulli(0.6) fill, largest 6-connected component,
    two materials per voxel (passive E=1e6; active E=1e6 with CTE=0.01), +-39 C
    at 5 Hz with expansion off, self-collision and floor on."""
    rng = np.random.default_rng(seed)
    mats = [Material(E=1e6, nu=0.35, cte=0.0, name="passive"), Material(E=1e6, nu=0.35, cte=0.01, name="active")]
    return [bernoulli_body(rng, (n, n, n), 0.6, mats, temp_vary=True, temp_amplitude=39.0, temp_period=0.2,
                           enable_collision=True)]


def c3_population(seed: int = 0, n_robots: int = 1024, lo: int = 4, hi: int = 16) -> List[Robot]:
    """Batched population: robots with dims uniform in [lo,hi]^3, Bernoulli(0.7),
    largest component, 4 materials with E log-uniform in [1e5,1e7] and CTE 0.01,
    per-voxel actuation phase uniform in [0, 2*pi) (stored in cycles), +-39 C at
    5 Hz, floor on, collisions off."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_robots):
        dims = tuple(int(x) for x in rng.integers(lo, hi + 1, size=3))
        mats = [Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, cte=0.01) for _ in range(4)]
        out.append(bernoulli_body(rng, dims, 0.7, mats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                                  temp_period=0.2))
    return out


def c4_differentiable(seed: int = 0) -> List[Robot]:
    """Differentiable single robot: 12x12x6 fully filled body, per-voxel actuation
    phase uniform in [0, 2*pi) (stored in cycles) and per-voxel log10 E uniform in
    [5, 7], 5 Hz actuation, floor friction on, no collisions."""
    rng = np.random.default_rng(seed)
    grid = np.ones((6, 12, 12), np.uint8)
    phase = rng.random((6, 12, 12)).astype(np.float32).astype(np.float64)
    log10E = rng.uniform(5, 7, size=(6, 12, 12)).astype(np.float32).astype(np.float64)
    m = Material(E=1e6, nu=0.35, rho=1e3, cte=0.01, mu_static=1.0, mu_kinetic=0.5)
    return [Robot(grid=grid, materials=[m], phase=phase, log10E=log10E, temp_vary=True, temp_amplitude=39.0,
                  temp_period=0.2)]


def c5_population_collisions(seed: int = 0, n_robots: int = 256) -> List[Robot]:
    """Collision-heavy population: 256 robots with dims uniform in [8,20]^3,
    Bernoulli(0.65), 4 materials, per-voxel phase, self-collision and floor on."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_robots):
        dims = tuple(int(x) for x in rng.integers(8, 21, size=3))
        mats = [Material(E=float(10 ** rng.uniform(5, 7)), nu=0.35, cte=0.01) for _ in range(4)]
        out.append(bernoulli_body(rng, dims, 0.65, mats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                                  temp_period=0.2, enable_collision=True))
    return out
