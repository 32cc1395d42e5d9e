"""FP64 adjoint of the step (vx3g_record / vx3g_backward) on the GPU, through the C ABI.

Workload: the differentiable single robot (12x12x6 full body, per-voxel phase in
[0, 2*pi) and per-voxel log10 E in [5, 7], 5 Hz actuation at 39 C with CTE 0.01,
floor friction), 2000 steps, checkpoint every 100.  Loss L = -(COM_x(T) - COM_x(0)).
Gradients are taken with respect to the phase in radians (the C ABI works in
cycles: d/d(rad) = d/d(cycles) / 2*pi) and log10 E.

The loss of this workload is only piecewise smooth: every friction stick/slip
event, contact change and small/large-angle switch of a link is a kink, and over
2000 steps they are dense enough in parameter space that a central difference
with eps = 1e-4 often straddles one (the estimate then moves by tens of percent
between eps = 1e-4, 1e-5 and 1e-6).  The adjoint is the derivative of the smooth
piece the run is on.  Tolerances (written here):
  * 32 seeded parameters (16 phases, 16 moduli; a modulus whose perturbation would
    change the stable dt is not drawn, the time step being held fixed), central
    differences at eps = 1e-4, 1e-5 and 1e-6: at least 24 of 32 agree with the
    adjoint within 3% at one of the three, and the median error at eps = 1e-6 is
    at most 5%.  (The single-step adjoint is checked exactly against finite
    differences on the host: tests/test_adjoint_host.py.)
  * checkpoint interval: gradients with K = 1, 7, 100 and N agree to 1e-12
    relative (the recompute is deterministic, the reverse sweep identical).
"""

import numpy as np
import pytest

from vx3g import abi
from vx3g import workloads as wl

pytestmark = pytest.mark.gpu

N_STEPS = 2000
EPS = (1e-4, 1e-5, 1e-6)


def _c4():
    return wl.c4_differentiable(0)[0]


def _with(base, phase=None, log10E=None):
    kw = dict(base.__dict__)
    if phase is not None:
        kw["phase"] = phase
    if log10E is not None:
        kw["log10E"] = log10E
    return wl.Robot(**kw)


def _loss(robot, n):
    b = abi.Batch([robot], abi.PRECISION_FP64)
    dt = b.dt()[0]
    c0 = b.com()[0, 0]
    b.step(n)
    out = -(b.com()[0, 0] - c0)
    b.close()
    return out, dt


def _gradient(robot, n, k=100):
    b = abi.Batch([robot], abi.PRECISION_FP64)
    b.record(n, k)
    gp, ge = b.backward(np.array([[-1.0, 0.0, 0.0]]))
    dt = b.dt()[0]
    b.close()
    return gp / (2 * np.pi), ge, dt


def fd_table(n=N_STEPS, eps_list=EPS, seed=1):
    """Adjoint and central differences on 32 seeded parameters: (adj[32], fd[len(eps), 32], kinds)."""
    base = _c4()
    gp, ge, dt0 = _gradient(base, n)
    nv = gp.size
    rng = np.random.default_rng(seed)
    ph = base.phase.reshape(-1)
    le = base.log10E.reshape(-1)
    lemax = np.sort(le)[-8:].min()
    vp = rng.choice(nv, 16, replace=False)
    ve = rng.choice(np.flatnonzero(le < lemax), 16, replace=False)
    adj = np.concatenate([gp[vp], ge[ve]])
    fd = np.zeros((len(eps_list), 32))
    for j, eps in enumerate(eps_list):
        for i, v in enumerate(vp):
            d = eps / (2 * np.pi)
            p1, p2 = ph.copy(), ph.copy()
            p1[v] += d
            p2[v] -= d
            f1, dt1 = _loss(_with(base, phase=p1.reshape(base.phase.shape)), n)
            f2, dt2 = _loss(_with(base, phase=p2.reshape(base.phase.shape)), n)
            assert dt1 == dt0 and dt2 == dt0
            fd[j, i] = (f1 - f2) / (2 * eps)
        for i, v in enumerate(ve):
            e1, e2 = le.copy(), le.copy()
            e1[v] += eps
            e2[v] -= eps
            f1, dt1 = _loss(_with(base, log10E=e1.reshape(base.log10E.shape)), n)
            f2, dt2 = _loss(_with(base, log10E=e2.reshape(base.log10E.shape)), n)
            assert dt1 == dt0 and dt2 == dt0
            fd[j, 16 + i] = (f1 - f2) / (2 * eps)
    return adj, fd, ["phase"] * 16 + ["log10E"] * 16


def rel_errors(adj, fd):
    scale = np.maximum(np.maximum(np.abs(fd), np.abs(adj)), 1e-2 * np.abs(adj).max())
    return np.abs(adj - fd) / scale


def test_adjoint_matches_central_fd():
    adj, fd, _ = fd_table()
    rel = rel_errors(adj, fd)
    best = rel.min(axis=0)
    assert np.sum(best <= 0.03) >= 24, (np.sort(best), rel)
    assert np.median(rel[EPS.index(1e-6)]) <= 0.05, rel


def test_checkpoint_interval_does_not_change_the_gradient():
    base = _c4()
    n = 300
    ref = _gradient(base, n, k=100)
    for k in (1, 7, n):
        g = _gradient(base, n, k=k)
        for a, b in zip(g[:2], ref[:2]):
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12 * np.abs(b).max())


def test_record_advances_like_step():
    base = _c4()
    a = abi.Batch([base], abi.PRECISION_FP64)
    b = abi.Batch([base], abi.PRECISION_FP64)
    a.record(250, 100)
    b.step(250)
    sa, sb = a.state(), b.state()
    for k in ("pos", "orient", "linmom", "angmom"):
        assert np.array_equal(sa[k], sb[k]), k
    a.backward(np.array([[1.0, 0.0, 0.0]]))  # the recorded end state is kept
    sc = a.state()
    for k in ("pos", "orient", "linmom", "angmom"):
        assert np.array_equal(sa[k], sc[k]), k
    assert a.steps_taken() == 250


def test_backward_needs_a_record_and_fp64():
    base = _c4()
    b = abi.Batch([base], abi.PRECISION_FP64)
    with pytest.raises(abi.Vx3gError, match="record"):
        b.backward(np.zeros((1, 3)))
    b.record(10, 5)
    b.step(1)  # the state no longer ends the recorded run
    with pytest.raises(abi.Vx3gError, match="record"):
        b.backward(np.zeros((1, 3)))
    m = abi.Batch([base], abi.PRECISION_MIXED)
    with pytest.raises(abi.Vx3gError, match="FP64"):
        m.record(10, 5)


def _contact_robot():
    """A self-colliding body with contacts from the first steps on: thermal expansion
    (EnableExpansion, 39 C, CTE 0.01) grows voxels to 1.39 voxel sizes, so diagonal
    neighbours (1.41 apart) fall inside the 1.25 x base-size contact envelope."""
    rng = np.random.default_rng(4)
    mats = [wl.Material(E=2e5, nu=0.35, cte=0.01), wl.Material(E=1e6, nu=0.35, cte=0.01)]
    r = wl.bernoulli_body(rng, (6, 5, 4), 0.85, mats, random_phase=True, temp_vary=True, temp_amplitude=39.0,
                          enable_collision=True, enable_expansion=1)
    log10E = np.where(r.grid > 0, rng.uniform(5.3, 6.0, size=r.grid.shape), 0.0).astype(np.float32).astype(np.float64)
    return wl.Robot(**{**r.__dict__, "log10E": log10E})


def test_collision_adjoint_matches_central_fd():
    """With voxel-voxel contact forces in the loop: 16 seeded parameters (8 phases,
    8 moduli) against central differences at eps = 1e-5 and 1e-6 over 150 steps;
    at least 12 of 16 within 3% at one of them."""
    base = _contact_robot()
    n = 150
    b = abi.Batch([base], abi.PRECISION_FP64)
    b.record(n, 50)
    assert np.count_nonzero(np.abs(b.voxel_aux()["contact"]).sum(1)) > 0  # contacts in play
    gp, ge = b.backward(np.array([[-1.0, 0.0, 0.0]]))
    gp = gp / (2 * np.pi)
    dt0 = b.dt()[0]
    b.close()
    grid = base.grid.reshape(-1) > 0
    ph = base.phase.reshape(-1)
    le = base.log10E.reshape(-1)
    idx = np.flatnonzero(grid)  # voxel order = lattice order of the filled cells
    rng = np.random.default_rng(2)
    pick = rng.choice(len(idx), 16, replace=False)
    lemax = np.sort(le[idx])[-4:].min()
    adj, fds = [], []
    for j, k in enumerate(pick):
        cell = idx[k]
        row = []
        for eps in (1e-5, 1e-6):
            if j < 8:
                d = eps / (2 * np.pi)
                p1, p2 = ph.copy(), ph.copy()
                p1[cell] += d
                p2[cell] -= d
                f1, d1 = _loss(_with(base, phase=p1.reshape(base.phase.shape)), n)
                f2, d2 = _loss(_with(base, phase=p2.reshape(base.phase.shape)), n)
            else:
                if le[cell] >= lemax:
                    break
                e1, e2 = le.copy(), le.copy()
                e1[cell] += eps
                e2[cell] -= eps
                f1, d1 = _loss(_with(base, log10E=e1.reshape(base.log10E.shape)), n)
                f2, d2 = _loss(_with(base, log10E=e2.reshape(base.log10E.shape)), n)
            assert d1 == dt0 and d2 == dt0
            row.append((f1 - f2) / (2 * eps))
        if len(row) < 2:
            continue
        adj.append(gp[k] if j < 8 else ge[k])
        fds.append(row)
    adj, fds = np.array(adj), np.array(fds).T
    rel = rel_errors(adj, fds)
    assert np.sum(rel.min(axis=0) <= 0.03) >= 0.75 * len(adj), (adj, fds, rel)


def test_torch_autograd_wrapper():
    torch = pytest.importorskip("torch")
    from adjoint_torch import COMDisplacement

    base = _c4()
    n = 150
    phase = torch.tensor(base.phase.reshape(-1) * 2 * np.pi, dtype=torch.float64, requires_grad=True)
    log10E = torch.tensor(base.log10E.reshape(-1), dtype=torch.float64, requires_grad=True)
    disp = COMDisplacement.apply(phase, log10E, base, n)
    loss = -disp[0]
    loss.backward()
    gp, ge, _ = _gradient(base, n)
    np.testing.assert_allclose(phase.grad.numpy(), gp, rtol=1e-12, atol=1e-20)
    np.testing.assert_allclose(log10E.grad.numpy(), ge, rtol=1e-12, atol=1e-20)
    f, _ = _loss(base, n)
    assert float(loss.detach()) == pytest.approx(f, rel=1e-12)
