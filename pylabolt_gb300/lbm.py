"""Python host object for one case on one GPU (wraps the C-ABI handle).

``FluidLBM(case)`` plays the role of the reference's operator set for the
fluidLB step (collision, force, compute-fields, streaming, boundary and
residue operators bound to one backend, pylabolt/solvers/fluidLB.py:109-204):
its methods are the calls the reference's ``Solver`` makes on them.
"""
import ctypes

import numpy as np

from . import capi
from .capi import check, ptr
from .config import Case
from .geometry import build_links

_STORAGE = {"fp64": capi.LBM_FP64, "fp32_shifted": capi.LBM_FP32_SHIFTED,
            "fp16_shifted": capi.LBM_FP16_SHIFTED}
_FORCING = {None: capi.LBM_FORCING_NONE, "guo_linear": capi.LBM_GUO_LINEAR,
            "guo_second_order": capi.LBM_GUO_SECOND_ORDER}


def make_config(case, storage=None, device=0, layout=None):
    storage = storage or case.storage
    layout = layout or case.population_layout
    cfg = capi.LbmConfig()
    cfg.nx, cfg.ny = case.nx, case.ny
    cfg.precision = _STORAGE[storage]
    cfg.collision = capi.LBM_MRT if case.collision == "MRT" else capi.LBM_BGK
    cfg.forcing = _FORCING[case.forcing]
    cfg.body_force_field = int(case.body_force_field is not None)
    cfg.device = device
    cfg.omega = case.omega
    cfg.inv_cs_2, cfg.inv_cs_4, cfg.eps = case.inv_cs_2, case.inv_cs_4, case.eps
    cfg.gravity[:] = [float(v) for v in case.gravity]
    cfg.mrt_s[:] = list(case.mrt_rates)
    cfg.fp16_scale = case.fp16_scale
    cfg.layout = capi.POP_AA if layout == "aa" else capi.POP_AB
    return cfg


def _is_tensor(a):
    return hasattr(a, "data_ptr") and hasattr(a, "is_cuda")


def _dptr(a):
    """ctypes pointer of a C-contiguous float64 array: a numpy array (host) or
    a torch tensor (host or CUDA; the C-ABI picks the copy direction)."""
    if _is_tensor(a):
        if not a.is_contiguous() or str(a.dtype) != "torch.float64":
            raise ValueError("tensor arguments must be contiguous float64")
        return ctypes.c_void_p(a.data_ptr())
    return ptr(a)


def _is_f32(a):
    """True for a float32 numpy array or torch tensor (the field type of a
    case with "precision": "single", pylabolt/base/fields.py:64-77)."""
    return str(a.dtype) in ("float32", "torch.float32")


def _fptr(a):
    """ctypes pointer of a C-contiguous float32 or float64 field, host or CUDA."""
    if _is_tensor(a):
        if not a.is_contiguous() or str(a.dtype) not in ("torch.float64", "torch.float32"):
            raise ValueError("tensor fields must be contiguous float64 or float32")
        return ctypes.c_void_p(a.data_ptr())
    if not a.flags.c_contiguous or a.dtype not in (np.float64, np.float32):
        raise ValueError("fields must be C-contiguous float64 or float32 arrays")
    return ptr(a)


class FluidLBM:
    """One fluidLB case resident on the GPU."""

    def __init__(self, case, storage=None, device=0, layout=None, body_force=None):
        if not isinstance(case, Case):
            case = Case(case)
        self.case = case
        self.storage = storage or case.storage
        self.layout = layout or case.population_layout
        if self.layout not in ("ab", "aa"):
            raise ValueError(f"unknown population layout {self.layout!r}")
        self.lib = capi.load()
        self.cfg = make_config(case, self.storage, device, self.layout)
        self.node_solid, self.links = build_links(case)
        h = ctypes.c_void_p()
        check(self.lib.lbm_create(ctypes.byref(self.cfg), ptr(self.node_solid),
                                  ptr(self.links), len(self.links), ctypes.byref(h)))
        self.h = h
        if case.body_force_field is not None:
            # body_force: the same field as an array or tensor (e.g. on the GPU)
            self.set_body_force(case.body_force_field if body_force is None else body_force)
        if case.moving:
            arr = (capi.LbmMovingObstacle * len(case.moving))()
            for a, o in zip(arr, case.moving):
                a.center[:] = [float(o.center[0]), float(o.center[1])]
                if o.type == "ellipse":
                    a.shape = 1
                    a.semi_axes[:] = [float(o.semi_axes[0]), float(o.semi_axes[1])]
                    a.radius = max(a.semi_axes[0], a.semi_axes[1])
                else:
                    a.radius = float(o.radius)
                a.velocity[:] = [float(o.linear_velocity[0]), float(o.linear_velocity[1])]
                a.omega = float(o.angular_velocity)
                # an ellipse starts at its inclination (degrees in obstacle_dict)
                a.angle = (float(np.float64(o.inclination) * np.pi / 180)
                           if o.type == "ellipse" else 0.0)
                a.mass = float(o.mass)
                a.inertia = float(o.moment_of_inertia)
                a.density = float(o.density)
                a.id = o.id
                a.calculated = int(o.calculated)
                a.rotation = int(o.rotation_allowed)
                a.translation = int(o.translation_allowed)
            g = (ctypes.c_double * 2)(*[float(v) for v in case.gravity])
            check(self.lib.lbm_set_moving_obstacles(self.h, arr, len(case.moving), g))

    # -- life cycle
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

    # -- set-up
    def initialize(self, density=None, velocity=None):
        """f = f_eq(rho, u) on fluid nodes (equilibrium_kernels.py:38-78).
        Float32 density and velocity (both; the fields of a single-precision
        case) cross the host link as float32 and are widened exactly on the
        device; anything else is taken as float64.  Contiguous CUDA tensors
        of either type are read on the device."""
        rho = self.case.density if density is None else density
        u = self.case.velocity if velocity is None else velocity
        n = self.case.nx * self.case.ny
        if _is_tensor(rho) and _is_tensor(u):
            if rho.dtype != u.dtype:
                raise ValueError("initialize: density and velocity of one dtype")
            if rho.is_cuda or u.is_cuda:
                import torch
                torch.cuda.current_stream(rho.device).synchronize()
            size = (rho.numel(), u.numel())
        else:
            if not (_is_f32(rho) and _is_f32(u)):
                rho = np.asarray(rho, dtype=np.float64)
                u = np.asarray(u, dtype=np.float64)
            rho = np.ascontiguousarray(rho)
            u = np.ascontiguousarray(u)
            size = (rho.size, u.size)
        if size != (n, 2 * n):
            raise ValueError("initialize: fields of the grid size")
        fn = self.lib.lbm_init_fields_f32 if _is_f32(rho) else self.lib.lbm_init_fields
        check(fn(self.h, _fptr(rho), _fptr(u), capi.LAYOUT_INNER))

    def set_body_force(self, force):
        """[Nx, Ny, 2] body-force field: a numpy array or a float64 torch
        tensor (a CUDA tensor is read on the device, after its stream)."""
        if _is_tensor(force):
            f = force.contiguous()
            if f.is_cuda:
                import torch
                torch.cuda.current_stream(f.device).synchronize()
        else:
            f = np.ascontiguousarray(force, dtype=np.float64)
        check(self.lib.lbm_set_body_force(self.h, _dptr(f)))

    # -- time stepping
    def step(self, nsteps=1, moments=False, residual=False):
        flags = (capi.STEP_MOMENTS if moments else 0) | (capi.STEP_RESIDUAL if residual else 0)
        check(self.lib.lbm_step_ex(self.h, int(nsteps), flags))

    def time_steps(self, nsteps):
        ms = ctypes.c_double()
        check(self.lib.lbm_time_steps(self.h, int(nsteps), ctypes.byref(ms)))
        return ms.value

    def synchronize(self, timeout_s=600.0):
        check(self.lib.lbm_synchronize(self.h, float(timeout_s)))

    # -- results
    def moments(self, layout=capi.LAYOUT_INNER, out=None, dtype=np.float64):
        """(rho, u) recorded at the last moments step: inner layout gives
        ``[Nx, Ny]`` / ``[Nx, Ny, 2]``; padded gives the reference's
        ``[(Nx+2)*(Ny+2)]`` / ``[..., 2]`` arrays (ghosts 0).  `dtype`
        float32 returns the fields of a single-precision case (each value
        rounded to nearest, exact for FP32/FP16 storage).  `out` = (rho, u):
        C-contiguous float64 or float32 arrays or tensors of that size to
        fill instead (e.g. pinned host memory for a faster copy)."""
        nx, ny = self.case.nx, self.case.ny
        n = nx * ny if layout == capi.LAYOUT_INNER else (nx + 2) * (ny + 2)
        if out is None:
            rho = np.empty(n, dtype=dtype)
            u = np.empty((n, 2), dtype=dtype)
        else:
            rho, u = out
            if _is_tensor(rho) and _is_tensor(u):   # e.g. CUDA tensors: filled on the device
                if rho.numel() != n or u.numel() != 2 * n or rho.dtype != u.dtype:
                    raise ValueError("moments(out=...): tensors of the grid size and one dtype")
                fn = self.lib.lbm_get_moments_f32 if _is_f32(rho) else self.lib.lbm_get_moments
                check(fn(self.h, _fptr(rho), _fptr(u), layout))
                if layout == capi.LAYOUT_INNER:
                    return rho.view(nx, ny), u.view(nx, ny, 2)
                return rho, u
            if (rho.dtype != u.dtype or rho.dtype not in (np.float64, np.float32) or rho.size != n
                    or u.size != 2 * n or not rho.flags.c_contiguous or not u.flags.c_contiguous):
                raise ValueError("moments(out=...): C-contiguous float64 or float32 arrays "
                                 "of the grid size")
        fn = self.lib.lbm_get_moments_f32 if _is_f32(rho) else self.lib.lbm_get_moments
        check(fn(self.h, _fptr(rho), _fptr(u), layout))
        if layout == capi.LAYOUT_INNER:
            return rho.reshape(nx, ny), u.reshape(nx, ny, 2)
        return rho, u

    def residual(self, step=None):
        """{res_rho, res_ux, res_uy} of the last residual step, or of the
        residual step that ended at time step `step` (one of the last eight):
        that form waits for that step only, so a loop can read step t's
        residual while step t + 1 runs."""
        out = (ctypes.c_double * 3)()
        if step is None:
            check(self.lib.lbm_residual(self.h, out))
        else:
            check(self.lib.lbm_residual_at(self.h, int(step), out))
        return np.array(out[:])

    def conservation(self):
        out = (ctypes.c_double * 3)()
        check(self.lib.lbm_conservation(self.h, out))
        return np.array(out[:])

    # -- momentum exchange (force_torque_kernels.py:11-141)
    def forces(self):
        """Force and torque from the momentum exchange on the current state:
        {"obstacles": [nobs, 3] (fx, fy, torque), "walls": [nwalls, 2]
        (fx, fy)}, in obstacle / wall-element order (``force_names``).  After
        ``initialize`` these are the t = 0 values."""
        if getattr(self, "_force_names", None) is None:
            from .obstacles import force_links
            links, obs, walls = force_links(self.case)
            ng = len(obs) + len(walls)
            links = np.ascontiguousarray(links)
            check(self.lib.lbm_set_force_links(self.h, ptr(links) if len(links) else None,
                                               len(links), ng))
            self._force_names = (obs, walls)
        obs, walls = self._force_names
        out = np.zeros((len(obs) + len(walls), 3))
        if len(out):
            check(self.lib.lbm_forces(self.h, ptr(out)))
        res = {"obstacles": out[:len(obs)], "walls": out[len(obs):, :2]}
        if self.case.moving:   # moving obstacles: the device's own momentum exchange
            full = np.zeros((len(self.case.obstacles), 3))
            static = [o for o in self.case.obstacles if o not in self.case.moving]
            for o, v in zip(static, res["obstacles"]):
                full[o.id] = v
            for st in self.moving_obstacles():
                full[st["id"]] = [st["force"][0], st["force"][1], st["torque"]]
            res["obstacles"] = full
        return res

    def moving_obstacles(self):
        """State of the moving obstacles: list of dicts (id, center, velocity,
        omega, angle, force, torque) in the case's moving-obstacle order."""
        n = len(self.case.moving)
        if n == 0:
            return []
        arr = (capi.LbmMovingObstacle * n)()
        check(self.lib.lbm_get_moving_obstacles(self.h, arr))
        return [{"id": a.id, "center": np.array(a.center[:]), "velocity": np.array(a.velocity[:]),
                 "omega": a.omega, "angle": a.angle, "force": np.array(a.force[:]),
                 "torque": a.torque} for a in arr]

    def node_flags(self):
        """[Nx, Ny] uint8: 0 fluid, 1 static solid, 2 + i solid of moving obstacle i."""
        out = np.empty(self.case.nx * self.case.ny, dtype=np.uint8)
        check(self.lib.lbm_get_node_flags(self.h, ptr(out)))
        return out.reshape(self.case.nx, self.case.ny)

    @property
    def force_names(self):
        """(obstacle names, wall element names) of ``forces``."""
        if getattr(self, "_force_names", None) is None:
            from .obstacles import force_links
            _, obs, walls = force_links(self.case)
            return obs, walls
        return self._force_names

    def populations(self):
        """Post-collision populations of the last step, padded AoS FP64."""
        nx, ny = self.case.nx, self.case.ny
        pop = np.empty(((nx + 2) * (ny + 2), 9))
        check(self.lib.lbm_get_populations(self.h, ptr(pop)))
        return pop

    def set_populations(self, pop_new):
        p = np.ascontiguousarray(pop_new, dtype=np.float64)
        check(self.lib.lbm_set_populations(self.h, ptr(p)))

    # -- adjoint (extension: the reference has no adjoint)
    def adjoint_forward(self, nsteps, interval=45):
        """Runs nsteps from the initialised fields, keeping a state every
        `interval` steps for the reverse pass; the last step's moments are
        recorded (:meth:`moments`)."""
        check(self.lib.lbm_adjoint_forward(self.h, int(nsteps), int(interval)))

    def adjoint_backward(self, grad_u, want_force=True):
        """Reverse pass for dL/du of the last step ([Nx, Ny, 2]).  Returns
        (dL/dF [Nx, Ny, 2] or None, dL/dtau, dL/du_wall [2]).  dL/du at solid
        nodes is ignored (their velocity is the body's, not computed).  A
        float64 CUDA tensor grad_u is read on the device, and dL/dF is then a
        CUDA tensor on the same device."""
        nx, ny = self.case.nx, self.case.ny
        want_f = want_force and self.case.body_force_field is not None
        if _is_tensor(grad_u) and grad_u.is_cuda:
            import torch
            gu = grad_u.detach().to(torch.float64).contiguous()
            torch.cuda.current_stream(gu.device).synchronize()
            gF = torch.empty((nx, ny, 2), dtype=torch.float64, device=gu.device) if want_f else None
        else:
            gu = np.ascontiguousarray(np.asarray(grad_u, dtype=np.float64).reshape(nx * ny, 2))
            gF = np.empty((nx, ny, 2)) if want_f else None
        gtau = ctypes.c_double()
        guw = (ctypes.c_double * 2)()
        check(self.lib.lbm_adjoint_backward(self.h, _dptr(gu), _dptr(gF) if gF is not None else None,
                                            ctypes.byref(gtau), guw))
        return gF, gtau.value, np.array(guw[:])

    # -- checkpoint / restart (lbm_save_state / lbm_load_state)
    def save_state(self):
        """The step state as a uint8 array (populations, boundary side data,
        residual history, time); `load_state` continues the run from it bit
        for bit in a handle of the same case."""
        n = ctypes.c_int64()
        check(self.lib.lbm_state_size(self.h, ctypes.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        check(self.lib.lbm_save_state(self.h, ptr(buf)))
        return buf

    def load_state(self, state):
        buf = np.ascontiguousarray(state, dtype=np.uint8)
        check(self.lib.lbm_load_state(self.h, ptr(buf)))

    @property
    def time(self):
        t = ctypes.c_int64()
        check(self.lib.lbm_time(self.h, ctypes.byref(t)))
        return t.value

    @property
    def kernel_launches(self):
        t = ctypes.c_int64()
        check(self.lib.lbm_kernel_launches(self.h, ctypes.byref(t)))
        return t.value

    @property
    def kernel_variant(self):
        """(kind, nodes per thread, threads per block, stages) of the fused
        step; kind 0 scalar, 2 node pairs from shared-memory tiles, 3 node pairs."""
        out = (ctypes.c_int * 4)()
        check(self.lib.lbm_kernel_variant(self.h, out))
        return tuple(out[:])

    @property
    def tuning(self):
        """Mean step time (ms) of every autotuner candidate."""
        out = (ctypes.c_double * 16)()
        n = ctypes.c_int()
        check(self.lib.lbm_tuning(self.h, out, ctypes.byref(n)))
        return list(out[:n.value])

    @property
    def device_bytes(self):
        t = ctypes.c_int64()
        check(self.lib.lbm_device_bytes(self.h, ctypes.byref(t)))
        return t.value
