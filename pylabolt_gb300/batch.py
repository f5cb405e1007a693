"""Many lid-driven cavities of uneven size and Reynolds number advanced as one
case: one fused kernel launch per time step for the whole batch (extension:
the reference runs one case per process).

The cavities are shelf-packed into one atlas grid.  Each cavity keeps its own
edge links: bounce-back walls, and a moving lid whose wall velocity sits in
its own link parameters (pylabolt/parallel/cpu/fluid_boundary_kernels.py:5-62
semantics, lid applied last).  Cells of the atlas outside every cavity are
solid and never touched.  Cavity x offsets are multiples of 32, so every
32-node row segment belongs to one cavity and carries that cavity's
relaxation rate (``lbm_set_omega_map``).  The result is an ordinary case for
the fused step kernel, so the launch-shape autotuner and the CUDA-graph replay
of ``lbm_step`` serve the batch unchanged.
"""
import ctypes

import numpy as np

from . import capi, workloads
from .capi import check, ptr, NODE_LINKS_DTYPE
from .config import Case
from .geometry import build_links


def draw_cavities(n=256, seed=0, side=(64, 512), re=(50.0, 1000.0), lid=(0.05, 0.1)):
    """Sides uniform in {64..512}, Re uniform in [50, 1000], lid velocity
    uniform in [0.05, 0.1], all from numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(side[0], side[1] + 1, size=n)
    res = rng.uniform(re[0], re[1], size=n)
    lids = rng.uniform(lid[0], lid[1], size=n)
    return sides, res, lids


def shelf_pack(sides, width, align=32):
    """Places squares of the given sides left to right on shelves of the
    atlas width, tallest first; x offsets aligned to `align`.  Returns
    (offsets [n, 2], atlas height)."""
    order = np.argsort(-np.asarray(sides), kind="stable")
    off = np.zeros((len(sides), 2), dtype=np.int64)
    x = y = shelf_h = 0
    for i in order:
        s = int(sides[i])
        if x + s > width:
            y += shelf_h
            x = shelf_h = 0
        off[i] = (x, y)
        x = (x + s + align - 1) // align * align
        shelf_h = max(shelf_h, s)
    return off, y + shelf_h


class CavityBatch:
    """`sides`, `res`, `lids`: per-cavity side, Reynolds number and lid
    velocity; nu = U N / Re, tau = 3 nu + 1/2 (as workloads.cavity)."""

    def __init__(self, sides, res, lids, storage="fp32_shifted", width=8192, device=0):
        self.sides = np.asarray(sides, dtype=np.int64)
        self.res = np.asarray(res, dtype=np.float64)
        self.lids = np.asarray(lids, dtype=np.float64)
        self.storage = storage
        self.off, height = shelf_pack(self.sides, width)
        self.nx, self.ny = int(width), int(height)
        nx, ny = self.nx, self.ny
        solid = np.ones((nx, ny), dtype=bool)
        omega = np.ones((nx, ny))
        recs = []
        self.cases = []
        for i, (n, re_i, u_i) in enumerate(zip(self.sides, self.res, self.lids)):
            case = Case(workloads.cavity(int(n), re=float(re_i), lid=float(u_i)))
            self.cases.append(case)
            ox, oy = (int(v) for v in self.off[i])
            solid[ox:ox + n, oy:oy + n] = False
            omega[ox:ox + n, oy:oy + n] = case.omega
            _, rec = build_links(case)
            # cavity node x*n + y  ->  atlas node (x+ox)*ny + (y+oy)
            r = rec.copy()
            for field in ("node", "src", "aux"):
                v = r[field]
                r[field] = (v // n + ox) * ny + (v % n + oy)
            recs.append(r)
        self.records = np.concatenate(recs)
        self.records.sort(order="node")
        self.node_solid = np.ascontiguousarray(solid.astype(np.uint8).ravel())
        self.fluid_nodes = int((~solid).sum())
        base = self.cases[0]
        cfg = capi.LbmConfig()
        cfg.nx, cfg.ny = nx, ny
        cfg.precision = {"fp64": capi.LBM_FP64, "fp32_shifted": capi.LBM_FP32_SHIFTED,
                         "fp16_shifted": capi.LBM_FP16_SHIFTED}[storage]
        cfg.collision, cfg.forcing = capi.LBM_BGK, capi.LBM_FORCING_NONE
        cfg.device = device
        cfg.omega = float(np.median([c.omega for c in self.cases]))
        cfg.inv_cs_2, cfg.inv_cs_4, cfg.eps = base.inv_cs_2, base.inv_cs_4, base.eps
        cfg.fp16_scale = base.fp16_scale
        self.lib = capi.load()
        h = ctypes.c_void_p()
        check(self.lib.lbm_create(ctypes.byref(cfg), ptr(self.node_solid), ptr(self.records),
                                  len(self.records), ctypes.byref(h)))
        self.h = h
        om = np.ascontiguousarray(omega.ravel())
        check(self.lib.lbm_set_omega_map(self.h, ptr(om)))

    def initialize(self):
        rho = np.ones(self.nx * self.ny)
        u = np.zeros((self.nx * self.ny, 2))
        check(self.lib.lbm_init_fields(self.h, ptr(rho), ptr(u), capi.LAYOUT_INNER))

    def step(self, nsteps, moments=False):
        check(self.lib.lbm_step_ex(self.h, int(nsteps), capi.STEP_MOMENTS if moments else 0))

    def time_steps(self, nsteps):
        ms = ctypes.c_double()
        check(self.lib.lbm_time_steps(self.h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def velocities(self):
        """Per-cavity velocity fields [n_i, n_i, 2] of the last moments step."""
        n = self.nx * self.ny
        rho = np.empty(n)
        u = np.empty((n, 2))
        check(self.lib.lbm_get_moments(self.h, ptr(rho), ptr(u), capi.LAYOUT_INNER))
        u = u.reshape(self.nx, self.ny, 2)
        return [u[ox:ox + s, oy:oy + s] for (ox, oy), s in zip(self.off, self.sides)]

    @property
    def kernel_variant(self):
        out = (ctypes.c_int * 4)()
        check(self.lib.lbm_kernel_variant(self.h, out))
        return tuple(out[:])

    def close(self):
        if getattr(self, "h", None):
            check(self.lib.lbm_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
