"""Test-only torch.autograd.Function around vx3g_record / vx3g_backward.

COMDisplacement.apply(phase_rad, log10E, robot, n_steps) runs the robot's FP64
step n_steps times with the given per-voxel phases (radians) and log10 Young's
moduli and returns its centre-of-mass displacement (3,); backward() maps dL/d(disp)
to dL/d(phase_rad), dL/d(log10E) through the hand-written adjoint (C ABI)."""

import numpy as np
import torch

from vx3g import abi
from vx3g import workloads as wl


class COMDisplacement(torch.autograd.Function):
    @staticmethod
    def forward(ctx, phase_rad, log10E, robot, n_steps, checkpoint_every=100):
        shape = robot.grid.shape
        ph = phase_rad.detach().cpu().numpy().astype(np.float64).reshape(shape) / (2 * np.pi)
        le = log10E.detach().cpu().numpy().astype(np.float64).reshape(shape)
        r = wl.Robot(**{**robot.__dict__, "phase": ph, "log10E": le})
        b = abi.Batch([r], abi.PRECISION_FP64)
        c0 = b.com()[0]
        b.record(int(n_steps), int(checkpoint_every))
        disp = b.com()[0] - c0
        ctx.batch = b
        return torch.tensor(disp, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_disp):
        w = grad_disp.detach().cpu().numpy().astype(np.float64).reshape(1, 3)
        gp, ge = ctx.batch.backward(w)
        ctx.batch.close()
        return (torch.from_numpy(gp / (2 * np.pi)), torch.from_numpy(ge), None, None, None)
