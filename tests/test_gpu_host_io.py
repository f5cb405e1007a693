"""Host transfers: by default a staging copy and a transposing kernel; with
LBM_HOST_DIRECT=1 the transposing kernels read and write pinned caller
buffers directly over the host link (where the device can reach host memory).
All routes must give the same bits."""
import numpy as np
import pytest
import torch

from _golden import load_golden
from pylabolt_gb300 import capi, workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu


def _pinned(a):
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
    t[...] = a
    return t


@pytest.mark.parametrize("storage", ["fp64", "fp32_shifted"])
@pytest.mark.parametrize("shape", [(200, 97), (64, 64)])
def test_pinned_and_pageable_routes_agree(storage, shape, monkeypatch):
    nx, ny = shape
    case = Case(workloads.cylinder(nx=nx, ny=ny, radius=8.0, center=(nx // 4, ny // 2 + 1)))
    rng = np.random.default_rng(5)
    rho = 1.0 + 1e-3 * rng.standard_normal((nx, ny))
    u = 1e-3 * rng.standard_normal((nx, ny, 2))
    out = {}
    for route in ("pageable", "pinned", "direct"):
        if route == "direct":
            monkeypatch.setenv("LBM_HOST_DIRECT", "1")
        with FluidLBM(case, storage=storage) as sim:
            if route == "pageable":
                sim.initialize(rho, u)
            else:
                sim.initialize(_pinned(rho), _pinned(u))
            sim.step(7, moments=True)
            if route == "pageable":
                r, v = sim.moments()
            else:
                r, v = sim.moments(out=(_pinned(np.zeros(nx * ny)), _pinned(np.zeros((nx * ny, 2)))))
            rp, vp = sim.moments(layout=capi.LAYOUT_PADDED)
            out[route] = (r.copy(), v.copy(), rp, vp, sim.populations())
    for route in ("pinned", "direct"):
        for a, b in zip(out[route], out["pageable"]):
            assert np.array_equal(a, b), route


def test_padded_initial_fields_pinned():
    case_d, d = load_golden("channel_cylinder_abb")
    case = Case(case_d)
    nx, ny = case.nx, case.ny
    rho_p = np.zeros((nx + 2) * (ny + 2))
    u_p = np.zeros(((nx + 2) * (ny + 2), 2))
    inner = np.zeros((nx + 2, ny + 2), bool)
    inner[1:-1, 1:-1] = True
    rho_p[inner.ravel()] = case.density.ravel()
    u_p[inner.ravel()] = case.velocity.reshape(-1, 2)
    with FluidLBM(case, storage="fp64") as a, FluidLBM(case, storage="fp64") as b:
        a.initialize()
        check = capi.check
        check(b.lib.lbm_init_fields(b.h, capi.ptr(_pinned(rho_p)), capi.ptr(_pinned(u_p)),
                                    capi.LAYOUT_PADDED))
        a.step(5)
        b.step(5)
        assert np.array_equal(a.populations(), b.populations())


def _pinned32(a):
    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True).numpy()
    t[...] = a
    return t


@pytest.mark.parametrize("storage", ["fp64", "fp32_shifted", "fp16_shifted"])
@pytest.mark.parametrize("route", ["pageable", "pinned", "direct", "cuda"])
def test_single_precision_fields(storage, route, monkeypatch):
    """lbm_init_fields_f32 gives the state lbm_init_fields gives on the same
    values as doubles; lbm_get_moments_f32 returns lbm_get_moments rounded to
    float32 (the fields of a "precision": "single" case), in both layouts."""
    nx, ny = 200, 97
    case = Case(workloads.cylinder(nx=nx, ny=ny, radius=8.0, center=(nx // 4, ny // 2 + 1)))
    rng = np.random.default_rng(11)
    rho = (1.0 + 1e-3 * rng.standard_normal((nx, ny))).astype(np.float32)
    u = (1e-3 * rng.standard_normal((nx, ny, 2))).astype(np.float32)
    if route == "direct":
        monkeypatch.setenv("LBM_HOST_DIRECT", "1")
    with FluidLBM(case, storage=storage) as a, FluidLBM(case, storage=storage) as b:
        a.initialize(rho.astype(np.float64), u.astype(np.float64))
        if route == "pageable":
            b.initialize(rho, u)
        elif route == "cuda":
            b.initialize(torch.from_numpy(rho).cuda(), torch.from_numpy(u).cuda())
        else:
            b.initialize(_pinned32(rho), _pinned32(u))
        assert np.array_equal(a.populations(), b.populations())
        r64, u64 = b.moments()
        if route == "pageable":
            r32, u32 = b.moments(dtype=np.float32)
        elif route == "cuda":
            rt = torch.empty(nx * ny, dtype=torch.float32, device="cuda")
            ut = torch.empty(nx * ny * 2, dtype=torch.float32, device="cuda")
            r32, u32 = (t.cpu().numpy() for t in b.moments(out=(rt, ut)))
        else:
            r32, u32 = b.moments(out=(_pinned32(np.zeros(nx * ny)), _pinned32(np.zeros((nx * ny, 2)))))
        assert r32.dtype == np.float32 and u32.dtype == np.float32
        assert np.array_equal(np.asarray(r32).reshape(nx, ny), r64.astype(np.float32))
        assert np.array_equal(np.asarray(u32).reshape(nx, ny, 2), u64.astype(np.float32))
        a.step(9, moments=True)
        b.step(9, moments=True)
        r64, u64 = b.moments(layout=capi.LAYOUT_PADDED)
        r32, u32 = b.moments(layout=capi.LAYOUT_PADDED, dtype=np.float32)
        assert np.array_equal(r32, r64.astype(np.float32))
        assert np.array_equal(u32, u64.astype(np.float32))
        if storage != "fp64":   # FP32 moments: the float32 read is exact
            assert np.array_equal(r32.astype(np.float64), r64)
            assert np.array_equal(u32.astype(np.float64), u64)
        ra, ua = a.moments()
        rb, ub = b.moments()
        assert np.array_equal(ra, rb) and np.array_equal(ua, ub)


def test_single_precision_padded_initial_fields():
    case_d, d = load_golden("channel_cylinder_abb")
    case = Case(case_d)
    nx, ny = case.nx, case.ny
    rho_p = np.zeros((nx + 2) * (ny + 2), np.float32)
    u_p = np.zeros(((nx + 2) * (ny + 2), 2), np.float32)
    inner = np.zeros((nx + 2, ny + 2), bool)
    inner[1:-1, 1:-1] = True
    rho_p[inner.ravel()] = case.density.ravel()
    u_p[inner.ravel()] = case.velocity.reshape(-1, 2)
    with FluidLBM(case, storage="fp32_shifted") as a, FluidLBM(case, storage="fp32_shifted") as b:
        a.initialize(case.density.astype(np.float32).astype(np.float64),
                     case.velocity.astype(np.float32).astype(np.float64))
        capi.check(b.lib.lbm_init_fields_f32(b.h, capi.ptr(_pinned32(rho_p)), capi.ptr(_pinned32(u_p)),
                                             capi.LAYOUT_PADDED))
        a.step(5)
        b.step(5)
        assert np.array_equal(a.populations(), b.populations())


@pytest.mark.parametrize("storage,layout", [("fp64", "ab"), ("fp32_shifted", "ab"), ("fp32_shifted", "aa")])
def test_residual_read_while_the_next_step_runs(storage, layout):
    """lbm_residual_at(t) gives step t's residual (the one lbm_residual
    returns right after step t) after later steps have been queued, for the
    last eight residual steps; older or never-computed steps are refused,
    and re-initialisation forgets them."""
    case = Case(workloads.cylinder(nx=300, ny=120, radius=10.0, center=(80, 61)))
    with FluidLBM(case, storage=storage, layout=layout) as sim:
        sim.initialize()
        sync = []
        for _ in range(12):
            sim.step(1, residual=True)
            sync.append(sim.residual())
    with FluidLBM(case, storage=storage, layout=layout) as sim:
        sim.initialize()
        piped = []
        for t in range(1, 13):
            sim.step(1, residual=True)
            if t > 1:
                piped.append(sim.residual(step=t - 1))
        piped.append(sim.residual(step=12))
        for t in range(5, 13):                          # the ring keeps the last eight
            assert np.array_equal(sim.residual(step=t), sync[t - 1])
        sim.step(3)                                     # plain steps do not touch the ring
        assert np.array_equal(sim.residual(step=12), sync[11])
        for t in (0, 4, 13, 15):
            with pytest.raises(RuntimeError, match="residual steps"):
                sim.residual(step=t)
        sim.initialize()
        with pytest.raises(RuntimeError, match="residual steps"):
            sim.residual(step=12)
    for a, b in zip(piped, sync):
        assert np.array_equal(a, b)
