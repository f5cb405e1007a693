"""liblbm_gb300.so on the CPU: it builds, loads, exports every symbol that
include/lbm_gb300.h declares, and rejects bad arguments before touching a
device (no compute call is made here)."""
import ctypes
import os
import re

import numpy as np
import pytest

from pylabolt_gb300 import capi
from pylabolt_gb300.capi import LbmConfig, NODE_LINKS_DTYPE, ptr

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "include", "lbm_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(lbm_\w+)\s*\(", text, re.M)))


def test_header_and_binding_agree():
    assert declared_functions() == sorted(capi.EXPORTS)


def test_library_exports_every_declared_symbol(lbm_lib):
    for name in declared_functions():
        assert hasattr(lbm_lib, name), name


def test_struct_layouts():
    assert ctypes.sizeof(LbmConfig) == 120
    assert NODE_LINKS_DTYPE.itemsize == 240


def _cfg(nx=8, ny=6, omega=1.2):
    c = LbmConfig()
    c.nx, c.ny, c.omega = nx, ny, omega
    c.inv_cs_2, c.inv_cs_4, c.eps = 3.0, 9.0, 2.2e-16
    c.fp16_scale = 4096.0
    return c


def _create(lib, cfg, solid, rec):
    h = ctypes.c_void_p()
    rc = lib.lbm_create(ctypes.byref(cfg), ptr(solid), ptr(rec) if rec is not None else None,
                        0 if rec is None else len(rec), ctypes.byref(h))
    return rc, lib.lbm_last_error().decode()


@pytest.mark.parametrize("field,value,msg", [
    ("nx", 0, "grid"), ("precision", 7, "precision"), ("collision", 5, "collision"),
    ("forcing", 9, "forcing"), ("omega", 2.5, "omega"), ("omega", 0.0, "omega")])
def test_create_rejects_bad_config(lbm_lib, field, value, msg):
    cfg = _cfg()
    setattr(cfg, field, value)
    solid = np.zeros(8 * 6, np.uint8)
    rc, err = _create(lbm_lib, cfg, solid, None)
    assert rc == capi.LBM_ERR_ARG and msg in err


def test_create_rejects_bulk_node_on_edge(lbm_lib):
    """Without link records the edge nodes would read outside the grid."""
    rc, err = _create(lbm_lib, _cfg(), np.zeros(48, np.uint8), None)
    assert rc == capi.LBM_ERR_ARG and "no link record" in err


def test_create_rejects_bad_links(lbm_lib):
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.geometry import build_links
    from _golden import load_golden
    case = Case(load_golden("channel_cylinder_abb")[0])
    solid, rec = build_links(case)
    cfg = _cfg(case.nx, case.ny)
    bad = rec.copy()
    bad["src"][0, 1] = case.nx * case.ny + 5
    bad["type"][0, 1] = capi.LINK_PULL
    rc, err = _create(lbm_lib, cfg, solid, bad)
    assert rc == capi.LBM_ERR_ARG and "out of range" in err
    bad = rec.copy()
    abb = np.argwhere(bad["type"] == capi.LINK_ABB)[0]
    bad = np.delete(bad, np.nonzero(bad["node"] == bad["aux"][abb[0], abb[1]])[0])
    rc, err = _create(lbm_lib, cfg, solid, bad)
    assert rc == capi.LBM_ERR_ARG
    dup = np.concatenate([rec, rec[:1]])
    rc, err = _create(lbm_lib, cfg, solid, dup)
    assert rc == capi.LBM_ERR_ARG and "two link records" in err


def test_null_arguments(lbm_lib):
    assert lbm_lib.lbm_step(None, 1) == capi.LBM_ERR_ARG
    assert lbm_lib.lbm_destroy(None) == capi.LBM_ERR_ARG
    out = (ctypes.c_double * 3)()
    assert lbm_lib.lbm_residual(None, out) == capi.LBM_ERR_ARG


def test_forced_allocation_failure(lbm_lib, monkeypatch):
    """Host-side fault injection: the env hook makes every allocation fail."""
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.geometry import build_links
    from _golden import load_golden
    case = Case(load_golden("cavity_lid_last")[0])
    solid, rec = build_links(case)
    monkeypatch.setenv("LBM_FAIL_ALLOC", "1")
    rc, err = _create(lbm_lib, _cfg(case.nx, case.ny), solid, rec)
    assert rc == capi.LBM_ERR_ALLOC and "LBM_FAIL_ALLOC" in err
