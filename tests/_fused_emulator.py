"""NumPy emulation of the fused step's data flow (test helper).

It runs the same plan as the CUDA kernel -- post-collision state, bulk pulls,
link records for boundary nodes, side array of the previous step's moments,
no-pull first step -- with the FP64 reference-order arithmetic, so the link
table built by ``pylabolt_gb300.geometry`` and the step mapping can be checked
against the oracle without a GPU.  Only tests import it.
"""
import numpy as np

from pylabolt_gb300.capi import LINK_PULL, LINK_ZERO, LINK_BB, LINK_MBB, LINK_ABB
from pylabolt_gb300.lattice import CX, CY, W, INV
from pylabolt_gb300.geometry import build_links


class FusedEmulator:
    def __init__(self, case):
        self.case = case
        nx, ny = case.nx, case.ny
        self.node_solid, self.rec = build_links(case)
        self.solid = self.node_solid.astype(bool)
        self.n = nx * ny
        self.recmap = np.full(self.n, -1, dtype=np.int64)
        self.recmap[self.rec["node"]] = np.arange(len(self.rec))
        self.fluid = np.nonzero(~self.solid)[0]
        self.bulk = self.fluid[self.recmap[self.fluid] < 0]
        self.spec = self.rec["node"]
        self.fstar = np.zeros((self.n, 9))
        self.side = np.zeros((len(self.rec), 3))
        self.nopull = True
        self.raux = np.zeros((len(self.rec), 9), dtype=np.int64)
        abb = self.rec["type"] == LINK_ABB
        self.raux[abb] = self.recmap[self.rec["aux"][abb]]

    def initialize(self):
        c = self.case
        rho = c.density.ravel()
        ux = c.velocity[..., 0].ravel()
        uy = c.velocity[..., 1].ravel()
        i2, i4 = c.inv_cs_2, c.inv_cs_4
        u2 = ux * ux + uy * uy
        for k in range(9):
            cu = CX[k] * ux + CY[k] * uy
            self.fstar[:, k] = W[k] * rho * (1 + i2 * cu + 0.5 * i4 * cu * cu - 0.5 * i2 * u2)
        self.fstar[self.solid] = 0.0
        self.rho = rho.copy()
        self.u = np.stack([ux, uy], axis=1)
        self.nopull = True

    def _incoming(self):
        c = self.case
        ny = c.ny
        fin = np.zeros((self.n, 9))
        if self.nopull:
            fin[:] = self.fstar
            return fin
        b = self.bulk
        for k in range(9):
            fin[b, k] = self.fstar[b - CX[k] * ny - CY[k], k]
        s = self.spec
        fin[s, 0] = self.fstar[s, 0]
        i2, h2, h4 = c.inv_cs_2, 0.5 * c.inv_cs_2, 0.5 * c.inv_cs_4
        for k in range(1, 9):
            kb = INV[k]
            t = self.rec["type"][:, k]
            raw = self.fstar[s, kb]
            val = np.zeros(len(s))
            m = t == LINK_PULL
            val[m] = self.fstar[self.rec["src"][m, k], k]
            val[t == LINK_ZERO] = 0.0
            m = t == LINK_BB
            val[m] = raw[m]
            m = t == LINK_MBB
            rho = self.side[m, 0]
            val[m] = raw[m] - ((2 * W[kb] * rho) * i2) * self.rec["param"][m, k]
            m = t == LINK_ABB
            if m.any():
                r = np.nonzero(m)[0]
                ra = self.raux[r, k]
                ux, uy = self.side[r, 1], self.side[r, 2]
                uex = ux + 0.5 * (ux - self.side[ra, 1])
                uey = uy + 0.5 * (uy - self.side[ra, 2])
                u2 = uex * uex + uey * uey
                cu = CX[kb] * uex + CY[kb] * uey
                temp = (2 * W[kb] * self.rec["param"][r, k]) * ((1 + (h4 * cu) * cu) - h2 * u2)
                val[r] = -raw[r] + temp
            fin[s, k] = val
        return fin

    def _active(self):
        """Nodes updated this step (fluid nodes)."""
        return self.fluid

    def step(self):
        c = self.case
        fin = self._incoming()
        idx = self._active()
        f = fin[idx]
        rho = np.zeros(idx.size)
        for k in range(9):
            rho = rho + f[:, k]
        if c.body_force_field is not None:
            Fx = c.body_force_field[..., 0].ravel()[idx]
            Fy = c.body_force_field[..., 1].ravel()[idx]
        else:
            Fx, Fy = rho * c.gravity[0], rho * c.gravity[1]
        sx = np.zeros(idx.size)
        sy = np.zeros(idx.size)
        for k in range(9):
            sx = sx + CX[k] * f[:, k]
            sy = sy + CY[k] * f[:, k]
        inv = 1 / (rho + c.eps)
        ux = sx * inv + 0.5 * Fx * inv
        uy = sy * inv + 0.5 * Fy * inv
        i2, i4, om = c.inv_cs_2, c.inv_cs_4, c.omega
        u2 = ux * ux + uy * uy
        out = np.zeros_like(f)
        for k in range(9):
            cu = CX[k] * ux + CY[k] * uy
            eq = W[k] * rho * (1 + i2 * cu + 0.5 * i4 * cu * cu - 0.5 * i2 * u2)
            v = (1 - om) * f[:, k] + om * eq
            if c.forcing == "guo_linear":
                v = v + (1 - 0.5 * om) * (W[k] * (CX[k] * Fx + CY[k] * Fy) * i2)
            elif c.forcing == "guo_second_order":
                cx_ = (CX[k] - ux) * i2 + cu * CX[k] * i4
                cy_ = (CY[k] - uy) * i2 + cu * CY[k] * i4
                v = v + (1 - 0.5 * om) * (W[k] * (cx_ * Fx + cy_ * Fy))
            out[:, k] = v
        self.fstar[idx] = out
        self.rho[idx] = rho
        self.u[idx, 0] = ux
        self.u[idx, 1] = uy
        self._after_collision(idx, rho)
        self.side[:, 0] = self.rho[self.spec]
        self.side[:, 1] = self.u[self.spec, 0]
        self.side[:, 2] = self.u[self.spec, 1]
        self.nopull = False

    def _after_collision(self, idx, rho):
        pass

    def padded(self, arr):
        """Inner x-major node array -> reference padded layout."""
        nx, ny = self.case.nx, self.case.ny
        a = np.asarray(arr).reshape((nx, ny) + np.asarray(arr).shape[1:])
        out = np.zeros((nx + 2, ny + 2) + a.shape[2:])
        out[1:-1, 1:-1] = a
        return out.reshape(((nx + 2) * (ny + 2),) + a.shape[2:])
