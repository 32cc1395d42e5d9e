"""The FP64 adjoint's algebra, checked on the host without a GPU.

tests/adjoint_host/adjoint_check.cpp compiles the product's step and adjoint
device functions (vx3g_step.cuh, vx3g_adjoint.cuh) as host C++ and compares them
with central finite differences of the same step:
  * "step": the vector-Jacobian product of one step at a state N steps into an
    actuated run (large-angle links, floor contact, damping active), with a random
    cotangent on every voxel and link state component; max error <= 1e-2 of
    (|fd| + 1% of the component class's largest |fd|), the finite-difference noise
    level at these step sizes;
  * "param": dCOM_x/d(phase) and dCOM_x/d(log10 E) over N steps against central
    differences with eps = 1e-4 on every voxel, short horizons where the loss is
    smooth; max error <= 5e-3 on the same scale.
"""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "adjoint_host", "adjoint_check.cpp")
CUDA_INC = "/usr/local/cuda/include"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path_factory.mktemp("adj") / "adjoint_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-w", "-I", CUDA_INC, "-x", "c++", SRC, "-o", exe],
                   check=True)
    return exe


def _run(exe, *args):
    out = subprocess.run([exe] + [str(a) for a in args], check=True, capture_output=True, text=True).stdout
    return {ln.split()[0]: float(ln.split()[1]) for ln in out.splitlines() if ln.strip()}


@pytest.mark.parametrize("n,dims", [(40, (3, 3, 2)), (300, (4, 3, 3))])
def test_one_step_vjp_matches_finite_differences(checker, n, dims):
    res = _run(checker, "step", n, *dims, 39.0)
    assert set(res) == {"pos", "quat", "linmom", "angmom", "link_state"}
    for k, e in res.items():
        assert e <= 1e-2, (k, e)


@pytest.mark.parametrize("n,floor", [(50, 1), (200, 0)])
def test_parameter_gradients_match_finite_differences(checker, n, floor):
    res = _run(checker, "param", n, 3, 3, 2, 39.0, floor)
    assert res["phase"] <= 5e-3 and res["log10E"] <= 5e-3, res
