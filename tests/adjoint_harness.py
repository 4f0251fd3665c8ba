"""Thin PyTorch harness over the engine's trajectory adjoint (C ABI
mps_trajectory_*): a torch.autograd.Function whose forward runs the
trajectory on the GPU and whose backward calls the hand-written adjoint.
PyTorch appears only here, in the tests."""
from __future__ import annotations

import numpy as np
import torch


class MpsTrajectoryFn(torch.autograd.Function):
    """(vel0 [n,3], gravity [3]) -> (sensor pressure [steps, sensors],
    final positions [n,3], final velocities [n,3]), all float64 on the CPU
    (the engine copies them in and out through host buffers)."""

    @staticmethod
    def forward(ctx, vel0, gravity, traj):
        sp, pos, vel = traj.forward(vel0.detach().numpy(), gravity.detach().numpy())
        ctx.traj = traj
        return torch.from_numpy(sp), torch.from_numpy(pos), torch.from_numpy(vel)

    @staticmethod
    def backward(ctx, d_sp, d_pos, d_vel):
        _, gv, gg = ctx.traj.backward(d_sp.contiguous().numpy(), d_pos.contiguous().numpy(),
                                      d_vel.contiguous().numpy())
        return torch.from_numpy(gv), torch.from_numpy(gg), None


def sensor_loss(sp):
    """Mean-squared pressure at the sensor particles over all steps."""
    return (sp ** 2).mean()


def position_loss(pos, target, fluid_mask):
    """Squared distance of the final fluid positions to a target."""
    return ((pos[fluid_mask] - target) ** 2).sum()


def wall_sensors(pos, types, l0, count=16):
    """The hydrostatic-tank pressure taps (mps_gb300.scenes.wall_taps)."""
    from mps_gb300 import scenes

    return scenes.wall_taps(pos, types, l0, count)
