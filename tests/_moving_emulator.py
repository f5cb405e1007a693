"""NumPy restatement of the moving-obstacle step (test helper, FP64).

It follows the device plan of pylabolt_gb300/csrc/lbm_moving.cuh operation by
operation -- motion of update_position_velocity, re-rasterisation, refill of
uncovered nodes, run-time moving-solid bounce-back of the nodes next to the
obstacle, the fixed-order momentum exchange -- on top of FusedEmulator's
fused-step plan, so the CUDA FP64 path can be compared with it bit for bit.
The reference's own moving path cannot run (obstacle_operator.py:67 calls an
undefined reconstruct_obstacles), so this restates the project's definition.
"""
import math

import numpy as np

from pylabolt_gb300.lattice import CX, CY, W, INV
from _fused_emulator import FusedEmulator


THREADS, BLOCKS = 256, 64   # the device's force launch (kMovForceThreads, kMovForceBlocks)


class MovingEmulator(FusedEmulator):
    def __init__(self, case):
        super().__init__(case)
        nx, ny = case.nx, case.ny
        self.cls_static = np.zeros(self.n, dtype=np.int64)
        self.cls_static[self.rec["node"]] = 1
        self.cls_static[self.solid] = 2
        self.gravity = np.asarray(case.gravity, dtype=np.float64)

    # -- set-up
    def initialize(self):
        super().initialize()
        c = self.case
        self.dsolid = np.zeros(self.n, dtype=np.int64)
        self.fresh = np.zeros(self.n, dtype=bool)
        self.us = np.zeros((self.n, 2))
        self.rho_dyn = self.rho.copy()
        self.cls = self.cls_static.copy()
        self.obs = []
        for o in c.moving:
            ell = o.type == "ellipse"
            self.obs.append({"cx": float(o.center[0]), "cy": float(o.center[1]),
                             "r": max(o.semi_axes) if ell else float(o.radius),
                             "shape": 1 if ell else 0,
                             "sa": float(o.semi_axes[0]) if ell else 0.0,
                             "sb": float(o.semi_axes[1]) if ell else 0.0,
                             "vx": float(o.linear_velocity[0]),
                             "vy": float(o.linear_velocity[1]), "om": float(o.angular_velocity),
                             "angle": float(np.float64(o.inclination) * np.pi / 180) if ell else 0.0,
                             "mass": float(o.mass),
                             "inertia": float(o.moment_of_inertia), "density": float(o.density),
                             "fx": 0.0, "fy": 0.0, "tq": 0.0, "calculated": o.calculated,
                             "rotation": o.rotation_allowed, "translation": o.translation_allowed})
        self._geometry(motion=False)
        self._forces(nopull=True)

    def _node(self, x, y):
        return x * self.case.ny + y

    # -- geometry of the coming step
    def _motion(self, o, motion):
        ncx, ncy = o["cx"], o["cy"]
        m = dict(o)
        if motion:
            om_old, vx_old, vy_old = o["om"], o["vx"], o["vy"]
            tt = fx = fy = 0.0
            if o["calculated"]:
                if o["rotation"]:
                    m["om"] = o["om"] + o["tq"] / o["inertia"]
                    tt = o["tq"]
                if o["translation"]:
                    m["vx"] = o["vx"] + (o["fx"] / o["mass"] + self.gravity[0])
                    m["vy"] = o["vy"] + (o["fy"] / o["mass"] + self.gravity[1])
                    fx, fy = o["fx"], o["fy"]
            if o["rotation"]:
                m["angle"] = o["angle"] + (om_old + 0.5 * tt / o["inertia"])
            if o["translation"]:
                ncx = o["cx"] + (vx_old + 0.5 * (fx / o["mass"] + self.gravity[0]))
                ncy = o["cy"] + (vy_old + 0.5 * (fy / o["mass"] + self.gravity[1]))
        assert abs(ncx - o["cx"]) < 1.0 and abs(ncy - o["cy"]) < 1.0
        r = o["r"]
        box = (math.floor(min(o["cx"], ncx) - r) - 1, math.ceil(max(o["cx"], ncx) + r) + 1,
               math.floor(min(o["cy"], ncy) - r) - 1, math.ceil(max(o["cy"], ncy) + r) + 1)
        nx, ny = self.case.nx, self.case.ny
        assert box[0] >= 2 and box[2] >= 2 and box[1] <= nx - 3 and box[3] <= ny - 3
        m["cx"], m["cy"], m["box"] = ncx, ncy, box
        if m["shape"] == 1:
            m["cth"], m["sth"] = math.cos(m["angle"]), math.sin(m["angle"])
        return m

    def _geometry(self, motion):
        self.obs = [self._motion(o, motion) for o in self.obs]
        for j, o in enumerate(self.obs):          # raster
            x0, x1, y0, y1 = o["box"]
            me = j + 1
            for x in range(x0, x1 + 1):
                for y in range(y0, y1 + 1):
                    n = self._node(x, y)
                    rx, ry = float(x) - o["cx"], float(y) - o["cy"]
                    if o["shape"] == 1:
                        xp = rx * o["cth"] + ry * o["sth"]
                        yp = -rx * o["sth"] + ry * o["cth"]
                        inside = (xp * xp) / (o["sa"] * o["sa"]) + (yp * yp) / (o["sb"] * o["sb"]) <= 1.0
                    else:
                        inside = rx * rx + ry * ry <= o["r"] * o["r"]
                    if inside:
                        self.dsolid[n] = me
                        ux, uy = o["vx"] - o["om"] * ry, o["vy"] + o["om"] * rx
                        self.us[n] = (ux, uy)
                        self.rho[n] = o["density"]
                        self.u[n] = (ux, uy)
                    elif self.dsolid[n] == me:
                        self.dsolid[n] = 0
                        self.fresh[n] = True
        ny = self.case.ny
        for j, o in enumerate(self.obs):          # classify + refill
            x0, x1, y0, y1 = o["box"]
            for x in range(x0 - 1, x1 + 2):
                for y in range(y0 - 1, y1 + 2):
                    n = self._node(x, y)
                    assert self.cls_static[n] == 0
                    if self.dsolid[n]:
                        self.cls[n] = 2
                        continue
                    nbs = [self._node(x + CX[k], y + CY[k]) for k in range(1, 9)]
                    self.cls[n] = 4 if any(self.dsolid[q] for q in nbs) else 0
                    if self.fresh[n]:
                        s, cnt = 0.0, 0
                        for q in nbs:
                            if self.dsolid[q] == 0 and not self.fresh[q]:
                                s += self.rho_dyn[q]
                                cnt += 1
                        rho = s / cnt if cnt else 1.0
                        self.fstar[n] = self._feq(rho, self.us[n, 0], self.us[n, 1])
                        self.rho_dyn[n] = rho

    def _feq(self, rho, ux, uy):
        c = self.case
        i2, i4 = c.inv_cs_2, c.inv_cs_4
        u2 = ux * ux + uy * uy
        out = np.zeros(9)
        for k in range(9):
            cu = CX[k] * ux + CY[k] * uy
            out[k] = W[k] * rho * (1 + i2 * cu + 0.5 * i4 * cu * cu - 0.5 * i2 * u2)
        return out

    # -- the fused step with class-4 nodes
    def _active(self):
        return np.nonzero((self.cls_static != 2) & (self.dsolid == 0))[0]

    def _incoming(self):
        fin = super()._incoming()
        if self.nopull:
            return fin
        c = self.case
        ny, i2 = c.ny, c.inv_cs_2
        for n in np.nonzero(self.cls == 4)[0]:
            x, y = divmod(int(n), ny)
            for k in range(1, 9):
                src = self._node(x - CX[k], y - CY[k])
                kb = INV[k]
                if self.dsolid[src]:
                    raw = self.fstar[n, kb]
                    cu = CX[kb] * self.us[src, 0] + CY[kb] * self.us[src, 1]
                    fin[n, k] = raw - ((2 * W[kb] * self.rho_dyn[n]) * i2) * cu
                else:
                    fin[n, k] = self.fstar[src, k]
        return fin

    def _after_collision(self, idx, rho):
        # the device keeps it for every node of a segment near the obstacle;
        # those are the only ones read, one step later
        self.rho_dyn[idx] = rho

    def step(self):
        self._geometry(motion=True)
        super().step()
        self._forces(nopull=False)

    # -- momentum exchange on each obstacle, the device's summation order:
    # thread g sums box nodes g, g + BLOCKS*THREADS, ..., a halving tree in
    # each block, then a halving tree over the blocks
    def _forces(self, nopull):
        c = self.case
        ny, i2 = c.ny, c.inv_cs_2
        for j, o in enumerate(self.obs):
            x0, x1, y0, y1 = o["box"]
            x0, y0 = x0 - 1, y0 - 1
            Wd, H = x1 - x0 + 2, y1 - y0 + 2
            lanes = np.zeros((BLOCKS * THREADS, 3))
            for i in range(Wd * H):
                x, y = x0 + i // H, y0 + i % H
                n = self._node(x, y)
                self.fresh[n] = False
                if self.cls[n] != 4:
                    continue
                first = 0
                for k in range(1, 9):
                    if first == 0:
                        first = self.dsolid[self._node(x + CX[k], y + CY[k])]
                if first != j + 1:
                    continue
                rx, ry = float(x) - o["cx"], float(y) - o["cy"]
                acc = lanes[i % (BLOCKS * THREADS)]
                for k in range(1, 9):
                    q = self._node(x + CX[k], y + CY[k])
                    if self.dsolid[q] == 0:
                        continue
                    kb = INV[k]
                    raw = self.fstar[n, k]
                    if nopull:
                        back = self.fstar[n, kb]
                    else:
                        cu = CX[k] * self.us[q, 0] + CY[k] * self.us[q, 1]
                        back = raw - ((2 * W[k] * self.rho_dyn[n]) * i2) * cu
                    vx = raw * CX[k] - back * CX[kb]
                    vy = raw * CY[k] - back * CY[kb]
                    acc[0] += vx
                    acc[1] += vy
                    acc[2] += rx * vy - ry * vx
            blk = lanes.reshape(BLOCKS, THREADS, 3)
            off = THREADS // 2
            while off:
                blk[:, :off] = blk[:, :off] + blk[:, off:2 * off]
                off //= 2
            lanes = blk[:, 0].copy()
            off = BLOCKS // 2
            while off:
                lanes[:off] = lanes[:off] + lanes[off:2 * off]
                off //= 2
            o["fx"], o["fy"], o["tq"] = lanes[0]
