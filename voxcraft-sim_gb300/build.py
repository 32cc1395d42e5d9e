"""Build libvx3g.so (the C-ABI library) in-tree with nvcc for sm_103a.

    python voxcraft-sim_gb300/build.py            # -> voxcraft-sim_gb300/_build/libvx3g.so

Translation units compile in parallel; the FP64 step and the auxiliary passes
use --fmad=false so that each multiply and add rounds on its own, as the
reference's arithmetic does.  The CUDA runtime is linked statically so the
library has no run-time path dependency.
"""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libvx3g.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr"]

UNITS = [
    ("vx3g_fp64.cu", ["--fmad=false"]),
    ("vx3g_aux.cu", ["--fmad=false"]),
    ("vx3g_attach.cu", ["--fmad=false"]),
    ("vx3g_mixed.cu", []),
    ("vx3g_adjoint.cu", ["--fmad=false"]),
    ("vx3g_host.cpp", []),
    ("vx3g_xml.cpp", []),
    ("vx3g_manager.cpp", []),
]
MAIN = "vx3g_sim_main.cpp"
EXE = os.path.join(OUT, "vx3g_sim")


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, unit + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(CSRC, u) for u, _ in UNITS + [(MAIN, [])]] + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                                                        if f.endswith((".h", ".cuh"))]
    srcs.append(os.path.join(os.path.dirname(HERE), "include", "vx3g.h"))
    srcs.append(os.path.join(os.path.dirname(HERE), "include", "vx3_simulation_manager.h"))
    newest = max(os.path.getmtime(s) for s in srcs)
    if not force and all(os.path.exists(p) and os.path.getmtime(p) >= newest for p in (LIB, EXE)):
        return LIB
    units = UNITS + [(MAIN, [])]
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        results = list(ex.map(lambda u: _compile(u[0], u[1], verbose), units))
    objs = [o for o, _ in results[:len(UNITS)]]
    main_obj = results[len(UNITS)][0]
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    cmd = [nvcc()] + ARCH + ["-cudart", "static", "-o", EXE, main_obj] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of vx3g_sim failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
