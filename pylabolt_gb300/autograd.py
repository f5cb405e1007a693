"""torch.autograd.Function over the GPU forward run and its hand-written
adjoint (extension: the reference has no differentiable path).

``lbm_velocity(case, force, tau, u_wall, nsteps)`` returns the velocity field
of the last step as a torch tensor; gradients flow to the body-force field
``force`` [Nx, Ny, 2], the relaxation time ``tau`` and the wall velocity
``u_wall`` [2] of the case's fixed_velocity boundaries.  The forward pass runs
on the GPU through the C-ABI (lbm_adjoint_forward), the backward pass is the
discrete adjoint (lbm_adjoint_backward) with checkpoint-and-recompute every
``interval`` steps.  PyTorch only carries the tensors and the graph.  CUDA
tensors stay on the device: the body-force field, the velocity, dL/du and
dL/dF pass through the C-ABI as device pointers, without a host round trip.
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
        on_gpu = force is not None and force.is_cuda
        if force is None:
            c = case_with(case, tau=float(tau), u_wall=u_wall.detach().cpu().numpy())
            sim = FluidLBM(c, storage=storage)
        elif on_gpu:
            # the case only needs to know that there is a body-force field;
            # its values come from the device tensor
            c = case_with(case, tau=float(tau), u_wall=u_wall.detach().cpu().numpy(),
                          force=np.zeros((case.nx, case.ny, 2)))
            f = force.detach().to(torch.float64).contiguous()
            sim = FluidLBM(c, storage=storage, device=f.device.index or 0, body_force=f)
        else:
            c = case_with(case, tau=float(tau), u_wall=u_wall.detach().cpu().numpy(),
                          force=force.detach().cpu().numpy())
            sim = FluidLBM(c, storage=storage)
        sim.initialize()
        sim.adjoint_forward(nsteps, interval)
        ctx.sim = sim
        ctx.has_force = force is not None
        ctx.devices = (force.device if force is not None else None, tau.device, u_wall.device)
        if on_gpu:
            n = case.nx * case.ny
            rho = torch.empty(n, dtype=torch.float64, device=force.device)
            u = torch.empty((n, 2), dtype=torch.float64, device=force.device)
            _, u = sim.moments(out=(rho, u))
            return u
        _, u = sim.moments()
        return torch.from_numpy(u).to(u_wall.device)

    @staticmethod
    def backward(ctx, grad_u):
        sim = ctx.sim
        dev_F, dev_tau, dev_uw = ctx.devices
        gF, gtau, guw = sim.adjoint_backward(grad_u if grad_u.is_cuda else grad_u.detach().cpu().numpy(),
                                              want_force=ctx.has_force)
        sim.close()
        if ctx.has_force and gF is not None:
            out_F = (gF if torch.is_tensor(gF) else torch.from_numpy(gF)).to(dev_F)
        else:
            out_F = None
        return (out_F, torch.tensor(gtau, dtype=torch.float64, device=dev_tau),
                torch.from_numpy(guw).to(dev_uw), None, None, None, None)


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
