"""Moving obstacles on the GPU against the CPU restatement of the same step
(tests/_moving_emulator.py), FP64 bit for bit: prescribed translation and
rotation, force-driven motion; plus the resting-obstacle identity with the
static path, FP32 against FP64, and the bounded failure when an obstacle
would leave its allowed region."""
import numpy as np
import pytest

from pylabolt_gb300 import capi
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM
from _moving_emulator import MovingEmulator
from test_moving_cpu import disk_case, wing_case

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-12


def _gpu(case, steps, storage="fp64"):
    with FluidLBM(case, storage=storage) as s:
        s.initialize()
        s.step(steps, moments=True)
        rho, u = s.moments()
        return rho, u, s.moving_obstacles(), s.node_flags()


def _emu(case, steps):
    e = MovingEmulator(case)
    e.initialize()
    for _ in range(steps):
        e.step()
    return e


@pytest.mark.parametrize("kw", [
    {"v": (0.05, 0.02), "om": 0.01},                       # prescribed translation + rotation
    {"v": (0.0, 0.0), "om": 0.0, "kind": "calculated", "density": 1.5},   # force-driven
])
def test_moving_disk_fp64_matches_restatement(kw):
    case = Case(disk_case(True, **kw))
    steps = 120
    rho, u, obs, flags = _gpu(case, steps)
    e = _emu(case, steps)
    nx, ny = case.nx, case.ny
    o, eo = obs[0], e.obs[0]
    assert o["center"][0] == eo["cx"] and o["center"][1] == eo["cy"]
    assert o["velocity"][0] == eo["vx"] and o["velocity"][1] == eo["vy"]
    assert o["omega"] == eo["om"] and o["angle"] == eo["angle"]
    assert o["force"][0] == eo["fx"] and o["force"][1] == eo["fy"] and o["torque"] == eo["tq"]
    assert np.array_equal(flags.ravel() >= 2, e.dsolid > 0)
    assert np.array_equal(rho.ravel(), e.rho)
    assert np.array_equal(u.reshape(-1, 2), e.u)


@pytest.mark.parametrize("kw", [
    {"v": (0.04, -0.02), "om": 0.015},                     # prescribed translation + rotation
    {"v": (0.0, 0.0), "om": 0.0, "kind": "calculated", "density": 1.2},   # force-driven
])
def test_moving_ellipse_fp64_matches_restatement(kw):
    """An inclined ellipse that translates and turns: the device raster in the
    frame of the angle the motion has reached, FP64 bit for bit against the
    restatement (positions, angle, forces, node flags, fields)."""
    case = Case(wing_case(True, **kw))
    steps = 120
    rho, u, obs, flags = _gpu(case, steps)
    e = _emu(case, steps)
    o, eo = obs[0], e.obs[0]
    assert o["center"][0] == eo["cx"] and o["center"][1] == eo["cy"]
    assert o["omega"] == eo["om"] and o["angle"] == eo["angle"]
    assert o["force"][0] == eo["fx"] and o["force"][1] == eo["fy"] and o["torque"] == eo["tq"]
    assert np.array_equal(flags.ravel() >= 2, e.dsolid > 0)
    assert np.array_equal(rho.ravel(), e.rho)
    assert np.array_equal(u.reshape(-1, 2), e.u)


def test_resting_moving_disk_equals_static_path():
    st_case = Case(disk_case(False))
    mv_case = Case(disk_case(True))
    with FluidLBM(st_case, storage="fp64") as s:
        s.initialize()
        f0 = s.forces()["obstacles"][0]
        s.step(200, moments=True)
        rho_s, u_s = s.moments()
        f_s = s.forces()["obstacles"][0]
    with FluidLBM(mv_case, storage="fp64") as m:
        m.initialize()
        g0 = m.forces()["obstacles"][0]
        m.step(200, moments=True)
        rho_m, u_m = m.moments()
        f_m = m.forces()["obstacles"][0]
    fl = ~st_case.solid
    fl &= ~mv_case.solid
    X, Y = np.meshgrid(np.arange(st_case.nx), np.arange(st_case.ny), indexing="ij")
    disk = (X - 14.0) ** 2 + (Y - 16.0) ** 2 <= 16.0
    fl &= ~disk
    assert np.array_equal(rho_s[fl], rho_m[fl]) and np.array_equal(u_s[fl], u_m[fl])
    np.testing.assert_allclose(g0, f0, rtol=FORCE_RTOL, atol=1e-15)
    np.testing.assert_allclose(f_m, f_s, rtol=FORCE_RTOL, atol=1e-15)


def test_moving_disk_fp32_close_to_fp64():
    case = Case(disk_case(True, v=(0.05, 0.02), om=0.01))
    _, u64, o64, _ = _gpu(case, 300)
    _, u32, o32, _ = _gpu(case, 300, storage="fp32_shifted")
    assert np.linalg.norm(u32 - u64) / np.linalg.norm(u64) <= 1e-5
    assert np.allclose(o32[0]["center"], o64[0]["center"], rtol=0, atol=1e-12)


def test_obstacle_leaving_its_region_fails_cleanly():
    case = Case(disk_case(True, v=(-0.5, 0.0), center=(9, 16)))
    with FluidLBM(case, storage="fp32_shifted") as s:
        s.initialize()
        with pytest.raises(capi.LbmError, match="within two nodes of the domain edge"):
            s.step(40)
            s.synchronize()
        # it stays where it last was allowed, and the handle keeps working
        c = s.moving_obstacles()[0]["center"][0]
        assert 7.0 <= c < 9.0
        s.step(1)


def test_registration_errors():
    """Host-side checks of lbm_set_moving_obstacles (no device work is done
    for a rejected set)."""
    with pytest.raises(capi.LbmError, match="two nodes away from the domain edges"):
        FluidLBM(Case(disk_case(True, center=(5, 16))))
    c = disk_case(True, center=(14, 16))
    c["obstacle_dict"]["wall_disk"] = {"type": "circle", "radius": 3.0, "center": [22, 16],
                                      "density": 1.0, "static": True}
    with pytest.raises(capi.LbmError, match="next to a boundary node or a static solid"):
        FluidLBM(Case(c))


def test_force_link_validation():
    case = Case(disk_case(False))
    with FluidLBM(case, storage="fp64") as s:
        links = np.zeros(1, dtype=capi.FORCE_LINK_DTYPE)
        links["node"] = 5 * case.ny + 5          # an interior bulk node: no link record
        links["k_out"], links["k_in"] = 1, 3
        with pytest.raises(capi.LbmError, match="not on a boundary node"):
            capi.check(s.lib.lbm_set_force_links(s.h, capi.ptr(links), 1, 1))
        links["node"] = 0
        links["group"] = 3
        with pytest.raises(capi.LbmError, match="group out of range"):
            capi.check(s.lib.lbm_set_force_links(s.h, capi.ptr(links), 1, 1))


@pytest.mark.parametrize("storage", ["fp64", "fp32_shifted"])
def test_residual_steps_do_not_change_the_moving_run(storage):
    """Residual steps run the residual instantiation of the moving-obstacle
    kernel, after a shape search whose trial launches must leave the state
    alone: the fields and the obstacle equal a run without residual steps
    (FP64 bit for bit; FP32 within one rounding per step, as for any two launch
    shapes)."""
    case = Case(disk_case(True, v=(0.05, 0.02), om=0.01))
    with FluidLBM(case, storage=storage) as a, FluidLBM(case, storage=storage) as b:
        a.initialize()
        b.initialize()
        for _ in range(4):
            a.step(10)
            a.step(5, residual=True)
            assert np.all(np.isfinite(a.residual()))
        b.step(60, moments=True)
        a.step(1, moments=True)
        b.step(1, moments=True)
        ra, ua = a.moments()
        rb, ub = b.moments()
        oa, ob = a.moving_obstacles()[0], b.moving_obstacles()[0]
        assert oa["center"][0] == ob["center"][0] and oa["center"][1] == ob["center"][1]
        if storage == "fp64":
            assert np.array_equal(ra, rb) and np.array_equal(ua, ub)
            assert np.array_equal(a.populations(), b.populations())
        else:
            assert np.abs(ua - ub).max() <= 1e-5 * np.abs(ub).max()
            assert np.abs(ra - rb).max() <= 1e-6


def _moving_channel(kind="fixed_velocity"):
    """A 512 x 128 channel (pressure-driven) with a cylinder of radius 12
    that translates and rotates (or moves under its forces): wide enough for
    whole bulk row segments around it."""
    from pylabolt_gb300 import workloads
    c = workloads.cylinder(nx=512, ny=128, radius=12.0, center=(160, 65))
    c["obstacle_dict"]["options"] = {"compute_force_torque": True, "move_obstacles": True}
    c["obstacle_dict"]["cylinder"].update({"static": False, "solid_motion_dict": {
        "type": kind, "degree_of_freedom": "both",
        "linear_velocity": [0.03, 0.01] if kind == "fixed_velocity" else [0.0, 0.0],
        "angular_velocity": 0.005 if kind == "fixed_velocity" else 0.0}})
    if kind == "calculated":
        c["obstacle_dict"]["cylinder"]["density"] = 1.5
    return Case(c)


@pytest.mark.parametrize("kind", ["fixed_velocity", "calculated"])
def test_moving_obstacles_on_the_node_pair_kernel(kind, monkeypatch):
    """The node-pair kernel serves cases with moving obstacles: bulk pairs on
    the fast path, the flagged segments around the obstacle on the per-node
    moving-obstacle path.  Against the scalar kernel, FP32, with residual and
    moment steps: the same obstacle track and fields within FP32 rounding."""
    case = _moving_channel(kind)
    out = []
    for v in ("0,1,128,1", "3,2,128,1"):
        monkeypatch.setenv("LBM_VARIANT", v)
        with FluidLBM(case, storage="fp32_shifted") as s:
            s.initialize()
            res = []
            for _ in range(4):
                s.step(40)
                s.step(10, residual=True)
                res.append(s.residual())
            s.step(1, moments=True)
            assert s.kernel_variant == tuple(int(i) for i in v.split(","))
            rho, u = s.moments()
            out.append((u, s.moving_obstacles()[0], np.array(res), s.node_flags()))
    (u0, o0, r0, f0), (u1, o1, r1, f1) = out
    fluid = ~case.solid
    assert np.abs(u1 - u0)[fluid].max() <= 1e-5 * np.abs(u0[fluid]).max()
    if kind == "fixed_velocity":
        assert o1["center"][0] == o0["center"][0] and o1["center"][1] == o0["center"][1]
        assert np.array_equal(f1, f0)
    else:
        assert np.allclose(o1["center"], o0["center"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(o1["force"], o0["force"], rtol=1e-4, atol=1e-9)
    np.testing.assert_allclose(r1, r0, rtol=1e-4)
