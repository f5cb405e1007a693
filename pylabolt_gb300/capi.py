"""ctypes bindings of liblbm_gb300.so (C-ABI: include/lbm_gb300.h).

The library is built in-tree by :mod:`pylabolt_gb300._build`.  There is no
fallback: if the shared library cannot be built or loaded, every call raises.
"""
import ctypes
import os

import numpy as np

from . import _build

LBM_OK, LBM_ERR_ARG, LBM_ERR_CUDA, LBM_ERR_NONFINITE = 0, 1, 2, 3
LBM_ERR_TIMEOUT, LBM_ERR_STATE, LBM_ERR_ALLOC = 4, 5, 6
LBM_FP64, LBM_FP32_SHIFTED, LBM_FP16_SHIFTED = 0, 1, 2
LBM_BGK, LBM_MRT = 0, 1
LBM_FORCING_NONE, LBM_GUO_LINEAR, LBM_GUO_SECOND_ORDER = 0, 1, 2
LINK_PULL, LINK_ZERO, LINK_BB, LINK_MBB, LINK_ABB = 0, 1, 2, 3, 4
LAYOUT_INNER, LAYOUT_PADDED = 0, 1
POP_AB, POP_AA = 0, 1
STEP_MOMENTS, STEP_RESIDUAL = 1, 2

STATUS_NAMES = {0: "LBM_OK", 1: "LBM_ERR_ARG", 2: "LBM_ERR_CUDA", 3: "LBM_ERR_NONFINITE",
                4: "LBM_ERR_TIMEOUT", 5: "LBM_ERR_STATE", 6: "LBM_ERR_ALLOC"}


class LbmError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class LbmNonFinite(LbmError):
    pass


class LbmConfig(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("collision", ctypes.c_int32),
                ("forcing", ctypes.c_int32), ("body_force_field", ctypes.c_int32),
                ("device", ctypes.c_int32), ("layout", ctypes.c_int32),
                ("omega", ctypes.c_double), ("inv_cs_2", ctypes.c_double),
                ("inv_cs_4", ctypes.c_double), ("eps", ctypes.c_double),
                ("gravity", ctypes.c_double * 2), ("mrt_s", ctypes.c_double * 4),
                ("fp16_scale", ctypes.c_double)]


class LbmMovingObstacle(ctypes.Structure):
    _fields_ = [("center", ctypes.c_double * 2), ("radius", ctypes.c_double),
                ("velocity", ctypes.c_double * 2), ("omega", ctypes.c_double),
                ("angle", ctypes.c_double), ("mass", ctypes.c_double),
                ("inertia", ctypes.c_double), ("density", ctypes.c_double),
                ("force", ctypes.c_double * 2), ("torque", ctypes.c_double),
                ("id", ctypes.c_int32), ("calculated", ctypes.c_int32),
                ("rotation", ctypes.c_int32), ("translation", ctypes.c_int32),
                ("semi_axes", ctypes.c_double * 2), ("shape", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class LbmPopView(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("pitch", ctypes.c_int64), ("plane", ctypes.c_int64),
                ("pop", ctypes.c_void_p), ("exclude", ctypes.c_void_p),
                ("fp16_scale", ctypes.c_double)]


NOALLOC_MAX_ROWS = 8192

# numpy mirror of LbmNodeLinks (must match the C struct byte for byte)
NODE_LINKS_DTYPE = np.dtype([("node", "<i8"), ("src", "<i8", 9), ("aux", "<i8", 9),
                             ("param", "<f8", 9), ("type", "i1", 9), ("wall", "i1"),
                             ("reserved", "i1", 6)])
assert NODE_LINKS_DTYPE.itemsize == 8 + 72 + 72 + 72 + 9 + 1 + 6

# numpy mirror of LbmForceLink
FORCE_LINK_DTYPE = np.dtype([("node", "<i8"), ("group", "<i4"), ("k_out", "i1"), ("k_in", "i1"),
                             ("reserved", "i1", 2), ("rx", "<f8"), ("ry", "<f8")])
assert FORCE_LINK_DTYPE.itemsize == 32

_LIB = None

# every symbol include/lbm_gb300.h declares
EXPORTS = ["lbm_create", "lbm_init_fields", "lbm_init_fields_f32", "lbm_set_body_force", "lbm_step",
           "lbm_step_ex", "lbm_get_moments", "lbm_get_moments_f32", "lbm_residual", "lbm_residual_at",
           "lbm_conservation",
           "lbm_get_populations", "lbm_set_populations", "lbm_time",
           "lbm_kernel_launches", "lbm_kernel_variant", "lbm_tuning", "lbm_device_bytes", "lbm_time_steps",
           "lbm_synchronize", "lbm_last_error", "lbm_destroy", "lbm_conservation_noalloc",
           "lbm_adjoint_forward", "lbm_adjoint_backward", "lbm_set_omega_map",
           "lbm_set_force_links", "lbm_forces", "lbm_set_moving_obstacles",
           "lbm_get_moving_obstacles", "lbm_get_node_flags", "lbm_state_size",
           "lbm_save_state", "lbm_load_state", "lbm_selftest_bounded_wait"]


def lib_path():
    return _build.LIB


def load(build=True):
    """Load (building first if needed) liblbm_gb300.so."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"liblbm_gb300.so not found at {path}")
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    i64 = ctypes.c_int64
    dbl = ctypes.POINTER(ctypes.c_double)
    sig = {
        "lbm_create": [ctypes.POINTER(LbmConfig), P, P, i64, ctypes.POINTER(P)],
        "lbm_init_fields": [P, P, P, ctypes.c_int],
        "lbm_init_fields_f32": [P, P, P, ctypes.c_int],
        "lbm_set_body_force": [P, P],
        "lbm_step": [P, i64],
        "lbm_step_ex": [P, i64, ctypes.c_int],
        "lbm_get_moments": [P, P, P, ctypes.c_int],
        "lbm_get_moments_f32": [P, P, P, ctypes.c_int],
        "lbm_residual": [P, dbl],
        "lbm_residual_at": [P, i64, dbl],
        "lbm_conservation": [P, dbl],
        "lbm_get_populations": [P, P],
        "lbm_set_populations": [P, P],
        "lbm_time": [P, ctypes.POINTER(i64)],
        "lbm_kernel_launches": [P, ctypes.POINTER(i64)],
        "lbm_device_bytes": [P, ctypes.POINTER(i64)],
        "lbm_kernel_variant": [P, ctypes.POINTER(ctypes.c_int)],
        "lbm_tuning": [P, dbl, ctypes.POINTER(ctypes.c_int)],
        "lbm_time_steps": [P, i64, dbl],
        "lbm_synchronize": [P, ctypes.c_double],
        "lbm_selftest_bounded_wait": [P, ctypes.c_double, dbl],
        "lbm_destroy": [P],
        "lbm_conservation_noalloc": [ctypes.POINTER(LbmPopView), P, P],
        "lbm_adjoint_forward": [P, i64, ctypes.c_int],
        "lbm_set_omega_map": [P, P],
        "lbm_adjoint_backward": [P, P, P, dbl, P],
        "lbm_set_force_links": [P, P, i64, ctypes.c_int],
        "lbm_forces": [P, P],
        "lbm_set_moving_obstacles": [P, P, ctypes.c_int, P],
        "lbm_get_moving_obstacles": [P, P],
        "lbm_get_node_flags": [P, P],
        "lbm_state_size": [P, ctypes.POINTER(i64)],
        "lbm_save_state": [P, P],
        "lbm_load_state": [P, P],
    }
    for name, argtypes in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_int
    lib.lbm_last_error.argtypes = []
    lib.lbm_last_error.restype = ctypes.c_char_p
    _LIB = lib
    return lib


def check(status):
    if status != LBM_OK:
        msg = load().lbm_last_error().decode(errors="replace")
        if status == LBM_ERR_NONFINITE:
            raise LbmNonFinite(status, msg)
        raise LbmError(status, msg)


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None
