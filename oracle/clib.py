"""ctypes driver for oracle/lbm_oracle.c (test infrastructure only).

``build()`` compiles the restatement with gcc into ``oracle/_build/``;
``COracle`` runs a case built by :func:`oracle.setup.build_state` through it.
"""
import ctypes
import os
import subprocess

import numpy as np

from .setup import W, INV_CS_2, INV_CS_4, EPS64
from .lbm_np import M_MRT, M_INV

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liblbm_oracle.so")
LIB_PATH_F32 = os.path.join(BUILD_DIR, "liblbm_oracle_f32.so")
SRC = os.path.join(HERE, "lbm_oracle.c")

BC_CODES = {"bounce_back": 0, "fixed_velocity": 1, "fixed_pressure": 2,
            "zero_gradient": 3}
FORCING_CODES = {None: 0, "guo_linear": 1, "guo_second_order": 2}


def build(force=False, real="double"):
    """Compile the C oracle (no fused multiply-add, OpenMP over nodes).
    real="float" builds the single-precision variant (float32 fields, the
    "precision": "single" case) used as a timed CPU baseline."""
    path = LIB_PATH if real == "double" else LIB_PATH_F32
    if (not force and os.path.exists(path)
            and os.path.getmtime(path) >= os.path.getmtime(SRC)):
        return path
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = path + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-fno-fast-math", "-ffp-contract=off",
                           "-fopenmp", "-fPIC", "-shared", f"-DOR_REAL={real}", SRC,
                           "-o", tmp, "-lm"])
    os.replace(tmp, path)
    return path


class OrParams(ctypes.Structure):
    _fields_ = [("nxp", ctypes.c_int64), ("nyp", ctypes.c_int64),
                ("collision", ctypes.c_int32), ("forcing", ctypes.c_int32),
                ("x_periodic", ctypes.c_int32), ("y_periodic", ctypes.c_int32),
                ("periodic_selfcopy", ctypes.c_int32), ("pad_", ctypes.c_int32),
                ("omega", ctypes.c_double), ("inv_cs_2", ctypes.c_double),
                ("inv_cs_4", ctypes.c_double), ("eps", ctypes.c_double),
                ("gravity", ctypes.c_double * 2), ("w", ctypes.c_double * 9),
                ("mrt_s", ctypes.c_double * 9), ("m", ctypes.c_double * 81),
                ("minv", ctypes.c_double * 81)]


class OrElement(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("normal", ctypes.c_int32 * 2),
                ("out_list", ctypes.c_int32 * 3), ("inv_list", ctypes.c_int32 * 3),
                ("pad_", ctypes.c_int32), ("value", ctypes.c_double * 2),
                ("node_begin", ctypes.c_int64), ("node_end", ctypes.c_int64)]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class COracle:
    """Holds a reference-layout state and advances it with the C oracle.
    real="float" runs the single-precision build on float32 copies of the
    state's fields (``self.f``); the default runs on the state itself."""

    def __init__(self, st, real="double"):
        self.lib = ctypes.CDLL(build(real=real))
        self.st = st
        self.real = real
        dt = np.float64 if real == "double" else np.float32
        self.f = {name: np.ascontiguousarray(getattr(st, name), dtype=dt) if real != "double"
                  else getattr(st, name)
                  for name in ("density", "velocity", "force", "pop", "pop_new")}
        p = OrParams()
        p.nxp, p.nyp = st.nxp, st.nyp
        p.collision = 1 if st.collision == "MRT" else 0
        p.forcing = FORCING_CODES[st.forcing]
        p.x_periodic, p.y_periodic = int(st.x_periodic), int(st.y_periodic)
        p.periodic_selfcopy = int(st.periodic_mode == "selfcopy")
        eps = EPS64 if real == "double" else float(np.finfo(np.float32).eps)
        p.omega, p.inv_cs_2, p.inv_cs_4, p.eps = st.omega, INV_CS_2, INV_CS_4, eps
        p.gravity[:] = list(st.gravity)
        p.w[:] = list(W)
        if st.mrt_rates is not None:
            s_e, s_eps, s_q, s_nu = st.mrt_rates
            p.mrt_s[:] = [1.0, s_e, s_eps, 1.0, s_q, 1.0, s_q, s_nu, s_nu]
        p.m[:] = list(M_MRT.ravel())
        p.minv[:] = list(M_INV.ravel())
        self.p = p
        self.idx = np.ascontiguousarray(np.nonzero(st.fluid)[0].astype(np.int64))
        self.solid = np.ascontiguousarray(st.solid.astype(np.uint8))
        els, nodes, pos = [], [], 0
        for el in st.elements:
            if el.type == "periodic":
                continue
            e = OrElement()
            e.type = BC_CODES[el.type]
            e.normal[:] = [int(v) for v in el.normal]
            e.out_list[:] = [int(v) for v in el.out_list]
            e.inv_list[:] = [int(v) for v in el.inv_list]
            if el.type == "fixed_velocity":
                e.value[:] = [float(v) for v in el.value]
            elif el.type == "fixed_pressure":
                e.value[0] = float(el.value)
            e.node_begin, e.node_end = pos, pos + el.nodes.size
            pos += el.nodes.size
            nodes.append(el.nodes)
            els.append(e)
        self.nel = len(els)
        self.els = (OrElement * max(1, self.nel))(*els)
        self.nodes = np.ascontiguousarray(
            np.concatenate(nodes) if nodes else np.zeros(1, np.int64)).astype(np.int64)
        self.body = (np.ascontiguousarray(st.body_force, dtype=dt)
                     if st.body_force is not None else None)
        self.density_old = np.zeros(st.size, dtype=dt)
        self.velocity_old = np.zeros((st.size, 2), dtype=dt)

    def initialize(self):
        f = self.f
        self.lib.or_initialize(ctypes.byref(self.p), _ptr(self.idx),
                               ctypes.c_int64(self.idx.size), _ptr(f["density"]),
                               _ptr(f["velocity"]), _ptr(f["pop"]), _ptr(f["pop_new"]))

    def run(self, nsteps):
        f = self.f
        self.lib.or_run(ctypes.byref(self.p), _ptr(self.idx),
                        ctypes.c_int64(self.idx.size), _ptr(self.solid),
                        _ptr(f["density"]), _ptr(f["velocity"]), _ptr(f["force"]),
                        _ptr(f["pop"]), _ptr(f["pop_new"]),
                        _ptr(self.body) if self.body is not None else None,
                        self.els, ctypes.c_int32(self.nel), _ptr(self.nodes),
                        ctypes.c_int64(nsteps))

    def residue(self):
        """Residuals (res_rho, res_ux, res_uy) -- pylabolt/utils/residues.py:171-222."""
        f = self.f
        out = np.zeros(6)
        self.lib.or_residue(_ptr(self.idx), ctypes.c_int64(self.idx.size),
                            _ptr(f["density"]), _ptr(f["velocity"]),
                            _ptr(self.density_old), _ptr(self.velocity_old), _ptr(out))
        return np.sqrt(out[0::2] / (out[1::2] + EPS64))
