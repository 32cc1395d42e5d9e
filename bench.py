"""Benchmark of the GB300 VX3 step: voxel-steps/s, mixed precision vs FP64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl vx3g|reference]
                    [--workload c2|c1|c3|c5] [--precision mixed|fp64]

The default line also carries the adjoint's backward/forward time ratio on the
differentiable 12x12x6 robot ("adjoint"; --no-adjoint leaves it out).

A bench "step" is --chunk (default 1000) physics time steps of the whole batch,
replayed as CUDA graphs of --graph-chunk (100) steps.  The timed run starts a fresh
context at physics step 0, so the default K (the configuration's steps / chunk: 20
for the single large body) covers the configuration's whole run; the W warm-up
bench steps run on a context of their own, which also tunes the launch shapes.
Timed steps are bracketed by CUDA events on the library's stream; the L2 cache is
flushed (512 MB overwrite) before every timed bench step.  The default workload is
the single large body (64^3 Bernoulli(0.6), collisions + floor, mixed precision).
Under torchrun each rank runs its own replica of the workload on its own GPU
(robots are independent; no collective).

The mixed-precision line also carries the metric's comparison: the FP64 step over
the same window ("fp64_value", "mixed_over_fp64"), the relative centre-of-mass error
of the mixed run against it ("com_rel_err", at 2000 steps and at the end of the
window), and the plain FP64 single-simulation rate of the 10^3 block
("c1_fp64_value").

"e2e" replays the same window on a fresh context through the C ABI with the voxel
state in pinned host memory: every bench step uploads the state, steps, reads the
state and the COM back.
"""

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from vx3g import abi, workloads  # noqa: E402

METRIC = "voxel-steps/s: mixed vs FP64 on GB300 at <=1e-5 rel COM err; bwd/fwd ratio"
UNIT = "voxel-steps/s"

WORKLOADS = {
    "c1": ("10x10x10 solid block drop, 1 robot, floor+friction, no collisions", workloads.c1_block_drop),
    "c2": ("64^3 Bernoulli(0.6) single body, 2 materials, 39C/5Hz actuation, self-collision + floor",
           workloads.c2_single_body),
    "c3": ("1024 robots [4,16]^3 Bernoulli(0.7), 4 materials, per-voxel phase, floor, no collisions",
           workloads.c3_population),
    "c5": ("256 robots [8,20]^3 Bernoulli(0.65), 4 materials, self-collision + floor", workloads.c5_population_collisions),
}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(nv, nl, ns, actuated, contacts=0):
    """Canonical bytes per physics step: link pass, voxel pass, collision."""
    link = 164 * nl + 56 * nv + (4 * nl if actuated else 0)
    voxel = 48 * nl + 240 * nv + (8 * nv if actuated else 0)
    coll = 48 * ns + 24 * contacts
    return dict(links=link, voxels=voxel, collision=coll)


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.proc, self.lines = device, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def barrier_and_max(value, world):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(value, world):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def init_dist(world):
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return dist
    return None


def cpu_baseline_port(robots, threads, budget_s=20.0, max_steps=200):
    """Time the oracle (the C restatement of the reference step, with the
    reference's all-pairs surface collision loop) on the host, on a bounded
    sample of the same workload: whole link+voxel steps of every robot for half
    the budget, and leading rows of each robot's all-pairs collision loop for
    the other half, scaled to the full S(S-1)/2 pairs.  Returns
    (voxel-steps/s, sample description)."""
    import oracle_bridge as ob
    sims = [ob.oracle_sim(r) for r in robots]
    for s in sims:
        s.set_threads(threads)
    nv = sum(s.counts()[0] for s in sims)
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        for s in sims:
            s.step_no_collision(1)
        steps += 1
        if time.perf_counter() - t0 > budget_s / 2:
            break
    t_lv = (time.perf_counter() - t0) / steps
    t_coll, rows_note = 0.0, ""
    coll = [(s, r) for s, r in zip(sims, robots) if r.enable_collision]
    if coll:
        per_robot_budget = budget_s / 2 / len(coll)
        done_pairs = total_pairs = 0
        for s, _ in coll:
            ns = s.counts()[2]
            pairs = ns * (ns - 1) / 2
            k, spent = 0, 0.0
            while k < ns and spent < per_robot_budget:
                k2 = min(ns, max(k + 64, int(k * 1.5)))
                spent += s.time_collision_rows(k, k2)
                k = k2
            done = k * (k - 1) / 2
            t_coll += spent * (pairs / done) if done else 0.0
            done_pairs += done
            total_pairs += pairs
        rows_note = f"; all-pairs collision timed on {done_pairs:.3g} of {total_pairs:.3g} surface pairs and scaled by pair count"
    per_step = t_lv + t_coll
    sample = (f"{steps} link+voxel step(s) of the full workload ({len(robots)} robot(s), {nv} voxels){rows_note}; "
              f"{threads} thread(s)")
    return nv / per_step, sample


def ncu_traffic(workload, precision, kernel):
    """DRAM bytes (read + write) per launch of `kernel` from the committed ncu summary
    of this workload (profiles/ncu_traffic.json), or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        return json.load(open(p))[f"{workload}/{precision}"][kernel]
    except (OSError, KeyError, ValueError):
        return None


def host_description():
    """CPU model and logical core count of the host the CPU baseline ran on."""
    model = ""
    try:
        for ln in open("/proc/cpuinfo"):
            k = ln.split(":")[0].strip().lower()
            if k in ("model name", "cpu model", "hardware") and ":" in ln:
                model = ln.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    if not model:
        import platform
        model = platform.processor() or platform.machine()
    return {"cpu": model, "nproc": os.cpu_count()}


def pinned_copy(arrays):
    """Copies of the arrays in page-locked host memory (torch's pinned allocator)."""
    try:
        import torch
        out = {}
        for k, a in arrays.items():
            t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
            t[...] = a
            out[k] = t
        return out
    except (ImportError, RuntimeError):
        return arrays


def measure_adjoint(dev, n=2000, k=100, reps=3):
    """Backward/forward time ratio on the differentiable 12x12x6 robot: FP64 forward
    of n steps (CUDA-graph chunks) vs vx3g_record (forward with checkpoints) and
    vx3g_backward (checkpoint recompute + reverse sweep), host wall clock around
    synchronised calls, best of `reps`."""
    robot = workloads.c4_differentiable(0)[0]
    fwd, rec, bwd = [], [], []
    for _ in range(reps):
        b = abi.Batch([robot], abi.PRECISION_FP64, device=dev)
        b.synchronize()
        t0 = time.perf_counter()
        b.step(n)
        b.synchronize()
        fwd.append(time.perf_counter() - t0)
        b.close()
        b = abi.Batch([robot], abi.PRECISION_FP64, device=dev)
        b.synchronize()
        t0 = time.perf_counter()
        b.record(n, k)
        b.synchronize()
        rec.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        b.backward(np.array([[-1.0, 0.0, 0.0]]))
        bwd.append(time.perf_counter() - t0)
        b.close()
    f, r, w = min(fwd), min(rec), min(bwd)
    return {"workload": "12x12x6 differentiable robot (864 voxels, per-voxel phase and log10 E), "
                        f"{n} FP64 steps, checkpoint every {k}",
            "fwd_fp64_ms": f * 1e3, "record_ms": r * 1e3, "backward_ms": w * 1e3,
            "bwd_over_fwd": w / f, "record_plus_bwd_over_fwd": (r + w) / f}


def measure_adjoint_population(dev, n=4000, k=100):
    """The batched differentiable population with collisions: the C5 robots with a
    per-voxel log10 E uniform in [5, 7] (fp32) added, FP64, n steps; the plain FP64
    batched forward (CUDA-graph chunks) vs vx3g_record + vx3g_backward (checkpoint
    every k).  Host wall clock around synchronised calls."""
    rng = np.random.default_rng(7)
    robots = []
    for r in workloads.c5_population_collisions():
        le = np.where(r.grid > 0, rng.uniform(5, 7, size=r.grid.shape), 0.0).astype(np.float32).astype(np.float64)
        robots.append(workloads.Robot(**{**r.__dict__, "log10E": le}))
    b = abi.Batch(robots, abi.PRECISION_FP64, device=dev)
    b.step(100)  # graphs built, lists warm
    b.synchronize()
    t0 = time.perf_counter()
    b.step(n)
    b.synchronize()
    fwd = time.perf_counter() - t0
    b.close()
    b = abi.Batch(robots, abi.PRECISION_FP64, device=dev)
    b.synchronize()
    t0 = time.perf_counter()
    b.record(n, k)
    b.synchronize()
    rec = time.perf_counter() - t0
    t0 = time.perf_counter()
    b.backward(np.tile(np.array([[-1.0, 0.0, 0.0]]), (len(robots), 1)))
    bwd = time.perf_counter() - t0
    nv = b.nv
    b.close()
    return {"workload": f"{len(robots)} robots [8,20]^3 Bernoulli(0.65), per-voxel phase and log10 E, "
                        f"self-collision + floor, {n} FP64 steps, checkpoint every {k}",
            "voxels": nv, "fwd_fp64_ms": fwd * 1e3, "record_ms": rec * 1e3, "backward_ms": bwd * 1e3,
            "bwd_over_fwd": bwd / fwd, "record_plus_bwd_over_fwd": (rec + bwd) / fwd,
            "gradient_entries_per_s": 2 * nv / (rec + bwd), "backward_voxel_steps_per_s": nv * n / bwd}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    builder = WORKLOADS[args.workload][1]
    robots = builder()
    cores = os.cpu_count() or 1
    value, sample = cpu_baseline_port(robots, cores, budget_s=args.ref_budget)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "config": {"workload": WORKLOADS[args.workload][0], "robots": len(robots)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                             "host": host_description()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# physics steps of each workload's configuration (the window one bench run covers)
CONFIG_STEPS = {"c1": 10000, "c2": 20000, "c3": 10000, "c5": 4000}


def timed_run(robots, prec, dev, K, C, G, cache, flush=True, com_at=()):
    """A fresh context of the workload from physics step 0: launch shapes from the tuning
    cache, step graphs captured beforehand, then K bench steps of C physics steps each,
    each between CUDA events on the library's stream (after a 512 MB L2 overwrite).
    Returns (per-step ms, context, {physics step: COM} for the steps in com_at)."""
    b = abi.Batch(robots, prec, device=dev, graph_chunk=G)
    b.autotune(0, cache)
    b.prepare_graphs()
    b.synchronize()
    ms, coms = [], {}
    for k in range(K):
        if flush:
            b.flush_l2()
        ms.append(b.time_steps(C))
        if (k + 1) * C in com_at:
            coms[(k + 1) * C] = b.com()
    return ms, b, coms


def profile_window(args):
    """The workload stepped to physics step START in CUDA graphs (launch shapes tuned
    first), then N steps with every kernel launched on its own, bracketed by the driver's
    profiler start and stop, so that a profiler started with collection off records only
    the kernels of those N steps (for a window deep into a run, e.g. C2's contact-heavy
    middle, without intercepting the launches before it)."""
    import ctypes
    start, n = args.profile_window
    robots = WORKLOADS[args.workload][1]()
    prec = abi.PRECISION_MIXED if args.precision == "mixed" else abi.PRECISION_FP64
    cache = args.tune_cache or os.path.join(tempfile.mkdtemp(prefix="vx3g_tune_"), "shapes.json")
    b = abi.Batch(robots, prec, device=0, graph_chunk=args.graph_chunk)
    b.autotune(min(start, 2000), cache)
    b.step(start - min(start, 2000))
    b.synchronize()
    cuda = ctypes.CDLL("libcuda.so.1")  # the context vx3g made current on this thread
    if cuda.cuProfilerStart() != 0:
        raise SystemExit("cuProfilerStart failed")
    for _ in range(n):
        b.step(1)  # a single step: its kernels launched one by one
    b.synchronize()
    cuda.cuProfilerStop()
    print(json.dumps({"profile_window": [start, n], "workload": args.workload, "precision": args.precision,
                      "steps_taken": int(b.steps_taken()), "status": [int(x) for x in b.status()]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="bench steps (default: the configuration's physics steps / --chunk, e.g. 20 for c2)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="vx3g", choices=["vx3g", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--chunk", type=int, default=1000, help="physics steps per bench step")
    ap.add_argument("--graph-chunk", type=int, default=100, help="physics steps per CUDA graph")
    ap.add_argument("--ref-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 run of the same window")
    ap.add_argument("--tune-cache", default=None, help="JSON cache of tuned launch shapes (read and appended)")
    ap.add_argument("--shard", action="store_true",
                    help="split the population across the ranks (robots [r*R/W, (r+1)*R/W) on rank r) "
                         "instead of one replica per rank")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch every step's kernels one by one instead of replaying CUDA graphs "
                         "(each launch then its own record in a per-kernel profiler)")
    ap.add_argument("--profile-window", type=int, nargs=2, metavar=("START", "N"), default=None,
                    help="for ncu --profile-from-start off: run START physics steps in CUDA graphs, then N "
                         "steps launched one by one between cuProfilerStart and cuProfilerStop; no bench line")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = max(1, CONFIG_STEPS[args.workload] // args.chunk)
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_window:
        return profile_window(args)

    rank, world, local = dist_env()
    dist = init_dist(world)
    dev = local
    desc, builder = WORKLOADS[args.workload]
    robots = builder()
    n_total = len(robots)
    if args.shard:  # this rank's contiguous range of the population; no data crosses ranks
        lo, hi = workloads.shard(len(robots), rank, world)
        robots = robots[lo:hi]
        if not robots:
            raise SystemExit(f"rank {rank}: no robots in its shard ({n_total} robots over {world} ranks)")
    prec = abi.PRECISION_MIXED if args.precision == "mixed" else abi.PRECISION_FP64
    W, K, C = args.warmup, args.steps, args.chunk
    G = -1 if args.no_graphs else args.graph_chunk
    cache = args.tune_cache or os.path.join(tempfile.mkdtemp(prefix="vx3g_tune_"), "shapes.json")
    actuated = any(r.temp_vary for r in robots)

    # warm-up on a context of its own: W bench steps, the first ones tuning the launch
    # shapes (written to the cache the timed contexts read), the clocks coming up
    bw = abi.Batch(robots, prec, device=dev, graph_chunk=G)
    tune = min(W * C, 2000)
    bw.autotune(tune, cache)
    if W * C > tune:
        bw.step(W * C - tune)
    bw.synchronize()
    bw.close()
    if dist:
        dist.barrier()
    com_at = {k * C for k in range(1, K + 1) if k * C in (2000, K * C)}
    with ClockSampler(dev) as clk:
        per_chunk, b, com_mx = timed_run(robots, prec, dev, K, C, G, cache, com_at=com_at)
    b.synchronize()
    if dist:
        dist.barrier()
    total_ms = barrier_and_max(float(np.sum(per_chunk)), world)
    status = b.status()
    nv, nl = b.nv, b.nl
    # units all ranks processed: replicas each step the whole workload; shards their ranges
    nv_job = allreduce_sum(float(nv), world) if args.shard else nv * world
    vox_steps = nv_job * C * K
    value = vox_steps / (total_ms / 1e3)
    surf = b.surface()
    ns_coll = 0
    global_grid = False  # some robot is listed on the global grid (k_grid_list launches every step)
    for i, r in enumerate(robots):
        if r.enable_collision:
            ns_r = int(np.count_nonzero((surf >= b.voxel_offset[i]) & (surf < b.voxel_offset[i + 1])))
            ns_coll += ns_r
            # the library lists a robot in shared memory when it has at most 6144 collision-surface
            # voxels and lattice coordinates below 512 (kLocalListMax)
            global_grid |= ns_r > 6144 or max(r.grid.shape) + r.z_offset > 512

    # per-pass device times (after the measured run); the dominant kernel is the single
    # kernel with the largest time: the link pass, the voxel pass or the contact evaluation
    passes = b.time_passes(20)
    ab = algorithmic_bytes(nv, nl, ns_coll, actuated)
    kernel_ms = {"k_links_mixed" if prec else "k_links": passes["links"],
                 "k_voxels_mixed" if prec else "k_voxels": passes["voxels"]}
    if ns_coll:
        kernel_ms["k_coll_eval_mixed" if prec else "k_coll_eval"] = passes["contact_eval"]
    kernel_bytes = dict(zip(kernel_ms, [ab["links"], ab["voxels"], ab["collision"]]))
    dom = max(kernel_ms, key=kernel_ms.get)
    peak, peak_kind = peaks()
    achieved = kernel_bytes[dom] / (kernel_ms[dom] / 1e3) / 1e9 if kernel_ms[dom] > 0 else 0.0
    traffic = ncu_traffic(args.workload, args.precision, dom)
    # link pass + voxel pass; collision: the displacement check, the cooperative list
    # rebuild kernel (it returns at once unless a rebuild is due), the global grid's list
    # kernel (the same) and the contact evaluation
    kernels_per_step = 2 + ((4 if global_grid else 3) if ns_coll else 0)
    shapes = [int(x) for x in b.launch_shapes()]
    b.close()

    # the metric's comparison: the FP64 step over the same window, and the mixed run's
    # relative COM error against it (end of the window, and at 2000 steps)
    fp64 = None
    if prec == abi.PRECISION_MIXED and not args.no_fp64:
        ms64, b64, com64 = timed_run(robots, abi.PRECISION_FP64, dev, K, C, G, cache, com_at=com_at)
        t64 = barrier_and_max(float(np.sum(ms64)), world)
        b64.close()
        rel = lambda a, c: np.linalg.norm(a - c, axis=1) / np.linalg.norm(c, axis=1)  # noqa: E731
        errs = {s: rel(com_mx[s], com64[s]) for s in sorted(com64)}
        fp64 = {"fp64_value": vox_steps / (t64 / 1e3), "fp64_ms_per_step": t64 / K,
                "mixed_over_fp64": (vox_steps / (total_ms / 1e3)) / (vox_steps / (t64 / 1e3)),
                "com_rel_err": {f"step_{s}": {"max": float(e.max()), "median": float(np.median(e)),
                                              "robots_le_1e-5": float(np.mean(e <= 1e-5))}
                                for s, e in errs.items()}}
        # the plain FP64 single-simulation step (the 10^3 block), the >= 3x denominator
        c1 = workloads.c1_block_drop()
        ms1, b1, _ = timed_run(c1, abi.PRECISION_FP64, dev, 2, 1000, G, cache, flush=False)
        fp64["c1_fp64_value"] = b1.nv * 1000 / (ms1[1] / 1e3)
        fp64["mixed_over_c1_fp64"] = value / fp64["c1_fp64_value"]
        b1.close()

    # e2e through the C ABI with host buffers: a fresh context of the same robots runs the
    # same K bench steps of the same trajectory from step 0, the voxel state living in
    # pinned host memory: every bench step uploads it, steps, reads it back and reads the COM
    b2 = abi.Batch(robots, prec, device=dev, graph_chunk=G)
    b2.autotune(0, cache)
    b2.prepare_graphs()
    host = pinned_copy(b2.state())
    b2.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(K):
        b2.set_state(**host)
        b2.step(C)
        b2.state(out=host)
        com = b2.com()
    e2e_s = barrier_and_max(time.perf_counter() - t0, world)
    h2d = sum(a.nbytes for a in host.values())
    d2h = h2d + com.nbytes
    e2e_value = nv_job * C * K / e2e_s
    b2.close()

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "strong" if args.shard else "weak",
        "vs_baseline": None,
        "dtype": "f32 link forces + f64 integration" if prec else "f64", "data": "synthetic (seeded generator)",
        "config": {"workload": desc, "robots": n_total, "robots_on_rank0": len(robots), "voxels": nv, "links": nl,
                   "collision_surface_voxels": ns_coll, "precision": args.precision,
                   "physics_steps_per_bench_step": C, "window": f"physics steps 0-{K * C} of a fresh context "
                   f"(the configuration runs {CONFIG_STEPS[args.workload]})",
                   "cuda_graphs": not args.no_graphs, "graph_chunk": G,
                   "launch_shapes": {"links": shapes[:2], "voxels": shapes[2:]},
                   "l2": "512 MB overwrite before every timed bench step",
                   "parallelism": f"robot shards x{world} of {n_total} robots" if args.shard else f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "kernel_ms": kernel_ms, "pass_ms": passes, "algorithmic_bytes_per_launch": ab,
                     # this GPU's algorithmic bytes over the job time, against one GPU's peak
                     "whole_step_algorithmic_gbs": (ab["links"] + ab["voxels"] + ab["collision"]) * C * K
                     / (total_ms / 1e3) / 1e9},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": kernels_per_step * C * K,
        "clocks": clk.summary(),
        "robot_status_nonzero": int(np.count_nonzero(status)),
    }
    if fp64:
        line.update(fp64)
    if rank == 0 and args.workload == "c2" and not args.no_adjoint:
        line["adjoint"] = measure_adjoint(dev)
    if rank == 0 and args.workload == "c5" and not args.no_adjoint:
        line["adjoint"] = measure_adjoint_population(dev)
    if rank == 0 and not args.no_cpu_baseline:
        # single-threaded, pinned to one core for the measurement
        pinned = None
        if hasattr(os, "sched_getaffinity"):
            pinned = os.sched_getaffinity(0)
            os.sched_setaffinity(0, {min(pinned)})
        try:
            v, sample = cpu_baseline_port(robots, 1, budget_s=15.0, max_steps=50)
        finally:
            if pinned is not None:
                os.sched_setaffinity(0, pinned)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample,
                                "host": host_description()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
