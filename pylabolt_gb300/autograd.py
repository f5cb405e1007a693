"""torch.autograd.Function over the GPU forward run and its hand-written
adjoint (extension: the reference has no differentiable path).

``lbm_velocity(case, force, tau, u_wall, nsteps)`` returns the velocity field
of the last step as a torch tensor; gradients flow to the body-force field
``force`` [Nx, Ny, 2], the relaxation time ``tau`` and the wall velocity
``u_wall`` [2] of the case's fixed_velocity boundaries.  The forward pass runs
on the GPU through the C-ABI (lbm_adjoint_forward), the backward pass is the
discrete adjoint (lbm_adjoint_backward) with checkpoint-and-recompute every
``interval`` steps.  PyTorch only carries the tensors and the graph.
"""
import copy

import numpy as np
import torch

from .config import Case
from .lbm import FluidLBM


def case_with(case, tau=None, u_wall=None, force=None):
    """A copy of `case` with another tau, wall velocity or body-force field."""
    c = copy.copy(case)
    if tau is not None:
        c.tau = float(tau)
        c.omega = float(1.0 / np.float64(c.tau))
        c.kin_visc = (c.tau - 0.5) / c.inv_cs_2
        c.mrt_rates = c.mrt_rates[:3] + (c.omega,)
    if u_wall is not None:
        c.elements = [copy.copy(e) for e in case.elements]
        for e in c.elements:
            if e.type == "fixed_velocity":
                e.value = [float(u_wall[0]), float(u_wall[1])]
    if force is not None:
        c.body_force_field = np.ascontiguousarray(force, dtype=np.float64)
    return c


class _LBMVelocity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, force, tau, u_wall, case, nsteps, interval, storage):
        c = case_with(case, tau=float(tau), u_wall=u_wall.detach().cpu().numpy(),
                      force=force.detach().cpu().numpy() if force is not None else None)
        sim = FluidLBM(c, storage=storage)
        sim.initialize()
        sim.adjoint_forward(nsteps, interval)
        _, u = sim.moments()
        ctx.sim = sim
        ctx.has_force = force is not None
        return torch.from_numpy(u).to(u_wall.device)

    @staticmethod
    def backward(ctx, grad_u):
        sim = ctx.sim
        gF, gtau, guw = sim.adjoint_backward(grad_u.detach().cpu().numpy(),
                                              want_force=ctx.has_force)
        sim.close()
        dev = grad_u.device
        out_F = torch.from_numpy(gF).to(dev) if (ctx.has_force and gF is not None) else None
        return (out_F, torch.tensor(gtau, dtype=torch.float64, device=dev),
                torch.from_numpy(guw).to(dev), None, None, None, None)


def lbm_velocity(case, force=None, tau=None, u_wall=None, nsteps=100, interval=45,
                 storage="fp32_shifted"):
    """Differentiable u of the last of `nsteps` steps (see module docstring)."""
    if not isinstance(case, Case):
        case = Case(case)
    if tau is None:
        tau = torch.tensor(case.tau, dtype=torch.float64)
    if u_wall is None:
        fv = [e for e in case.elements if e.type == "fixed_velocity"]
        u_wall = torch.tensor(fv[0].value if fv else [0.0, 0.0], dtype=torch.float64)
    return _LBMVelocity.apply(force, tau, u_wall, case, int(nsteps), int(interval), storage)
