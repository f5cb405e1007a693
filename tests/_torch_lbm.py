"""Plain-torch FP64 forward of the fluidLB step (BGK, Guo forcing, PULL /
ZERO / BB / MBB links), differentiable with torch.autograd.

It follows the same link table as the CUDA step (pylabolt_gb300.geometry) and
the reference step order, node by node, and is the FP64 reference gradient
for the hand-written adjoint.  Test helper only.
"""
import numpy as np
import torch

from pylabolt_gb300.capi import LINK_PULL, LINK_ZERO, LINK_BB, LINK_MBB, LINK_ABB
from pylabolt_gb300.geometry import build_links
from pylabolt_gb300.lattice import CX, CY, W, INV

FORCING = {None: 0, "guo_linear": 1, "guo_second_order": 2}


class TorchLBM:
    def __init__(self, case, dtype=torch.float64, device="cpu"):
        self.case = case
        self.dt = dtype
        self.dev = device
        nx, ny = case.nx, case.ny
        solid, rec = build_links(case)
        if np.any(rec["type"] == LINK_ABB):
            raise ValueError("anti-bounce-back is not differentiated here")
        n = nx * ny
        self.n = n
        self.fluid = torch.tensor(~solid.astype(bool), device=device)
        node = np.arange(n)
        x, y = node // ny, node % ny
        typ = np.full((n, 9), LINK_PULL, dtype=np.int64)
        src = np.zeros((n, 9), dtype=np.int64)
        par = np.zeros((n, 9))
        wall = np.zeros((n, 9), dtype=bool)
        for k in range(9):
            sx, sy = x - CX[k], y - CY[k]
            ok = (sx >= 0) & (sx < nx) & (sy >= 0) & (sy < ny)
            src[:, k] = np.where(ok, np.clip(sx, 0, nx - 1) * ny + np.clip(sy, 0, ny - 1), node)
        r = rec["node"]
        typ[r] = rec["type"]
        src[r] = np.where(rec["type"] == LINK_PULL, rec["src"], r[:, None])
        par[r] = rec["param"]
        wall[r] = (rec["wall"][:, None] != 0) & (rec["type"] == LINK_MBB)
        typ[:, 0] = LINK_PULL
        src[:, 0] = node
        t = torch.tensor
        self.typ = t(typ, device=device)
        self.src = t(src, device=device)
        self.par = t(par, dtype=dtype, device=device)
        self.wall = t(wall, device=device)
        self.cx = t(CX, dtype=dtype, device=device)
        self.cy = t(CY, dtype=dtype, device=device)
        self.w = t(W, dtype=dtype, device=device)
        self.inv = t(INV, device=device)
        self.i2 = t(case.inv_cs_2, dtype=dtype, device=device)
        self.i4 = t(case.inv_cs_4, dtype=dtype, device=device)
        self.forc = FORCING[case.forcing]

    def equilibrium(self, rho, ux, uy):
        cu = self.cx * ux[:, None] + self.cy * uy[:, None]
        u2 = (ux * ux + uy * uy)[:, None]
        return self.w * rho[:, None] * (1 + self.i2 * cu + 0.5 * self.i4 * cu * cu - 0.5 * self.i2 * u2)

    def run(self, nsteps, omega, force=None, u_wall=None):
        """Returns u of the last step [n, 2].  `force` [n, 2] is the body-force
        field (None: rho * gravity); `u_wall` [2] replaces the fixed_velocity
        links' wall velocity (their param = c_kbar . u_wall)."""
        c = self.case
        rho0 = torch.tensor(c.density.ravel(), dtype=self.dt, device=self.dev)
        u0 = torch.tensor(c.velocity.reshape(-1, 2), dtype=self.dt, device=self.dev)
        f = self.equilibrium(rho0, u0[:, 0], u0[:, 1])
        fl = self.fluid[:, None]
        f = torch.where(fl, f, torch.zeros_like(f))
        g = torch.tensor(c.gravity, dtype=self.dt, device=self.dev)
        par = self.par
        if u_wall is not None:
            kb = self.inv
            wall_par = self.cx[kb] * u_wall[0] + self.cy[kb] * u_wall[1]
            par = torch.where(self.wall, wall_par.expand_as(par), par)
        p = f
        rho_prev = None
        for t in range(1, nsteps + 1):
            if t == 1:
                fin = p
            else:
                raw = p[:, self.inv]                        # p(n)_kbar
                pulled = p.gather(0, self.src)              # p(src)_k  (column k)
                cols = []
                for k in range(9):
                    tk = self.typ[:, k]
                    v = torch.where(tk == LINK_PULL, pulled[:, k], torch.zeros_like(pulled[:, k]))
                    v = torch.where(tk == LINK_BB, raw[:, k], v)
                    mbb = raw[:, k] - 2 * self.w[self.inv[k]] * rho_prev * self.i2 * par[:, k]
                    v = torch.where(tk == LINK_MBB, mbb, v)
                    cols.append(v)
                fin = torch.stack(cols, 1)
            # solid nodes carry zeros: keep them away from 0/0 (their values
            # are discarded, but NaN would poison the gradient)
            rho = torch.where(self.fluid, fin.sum(1), torch.ones_like(fin[:, 0]))
            jx = (fin * self.cx).sum(1)
            jy = (fin * self.cy).sum(1)
            if self.forc == 0:
                Fx = Fy = torch.zeros_like(rho)
            elif force is not None:
                Fx, Fy = force[:, 0], force[:, 1]
            else:
                Fx, Fy = rho * g[0], rho * g[1]
            ux = (jx + 0.5 * Fx) / rho
            uy = (jy + 0.5 * Fy) / rho
            feq = self.equilibrium(rho, ux, uy)
            out = fin + omega * (feq - fin)
            if self.forc == 1:
                fbar = self.w * self.i2 * (self.cx * Fx[:, None] + self.cy * Fy[:, None])
                out = out + (1 - 0.5 * omega) * fbar
            elif self.forc == 2:
                cu = self.cx * ux[:, None] + self.cy * uy[:, None]
                ex = (self.cx - ux[:, None]) * self.i2 + cu * self.cx * self.i4
                ey = (self.cy - uy[:, None]) * self.i2 + cu * self.cy * self.i4
                fbar = self.w * (ex * Fx[:, None] + ey * Fy[:, None])
                out = out + (1 - 0.5 * omega) * fbar
            p = torch.where(fl, out, torch.zeros_like(out))
            rho_prev = rho
        return torch.stack([ux, uy], 1)
