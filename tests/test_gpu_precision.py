"""FP32 / FP16 shifted storage against FP64, MRT against the oracle, every
autotuner launch shape, and the large-case checks (full-size cavity bit-exact
against the C oracle, Poiseuille against the analytic start-up flow)."""
import os

import numpy as np
import pytest

from _golden import golden_names, load_golden
from pylabolt_gb300 import capi, workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

FP32_U_TOL = 1e-5     # max |u32 - u64| / max |u64|
# Start-up Poiseuille flow (1024x512, MRT + Guo, 50,000 steps): the flow
# grows by ~g = 4e-7 per step, and the exact-conservation relaxation keeps
# the FP32 rounding of that growth from accumulating (measured 1.2e-6 max,
# 6.1e-7 relative L2).  The bound is the 1e-5 stated for FP32 storage.
FP32_STARTUP_TOL = 1e-5
FP16_U_TOL = 2e-2
# FP64 MRT, CUDA closed form vs oracle matrix form: both round differently, so
# the bound is FP64 round-off accumulated over the run on O(1) populations.
MRT_ATOL = 1e-13


def _run(case, storage, steps, variant=None):
    old = os.environ.get("LBM_VARIANT")
    if variant:
        os.environ["LBM_VARIANT"] = ",".join(str(v) for v in variant)
    try:
        with FluidLBM(case, storage=storage) as sim:
            sim.initialize()
            sim.step(steps, moments=True)
            rho, u = sim.moments()
            return rho, u, sim.populations(), sim.kernel_variant
    finally:
        if variant:
            if old is None:
                del os.environ["LBM_VARIANT"]
            else:
                os.environ["LBM_VARIANT"] = old


def _rel(a, b, mask):
    return np.abs(a[mask] - b[mask]).max() / max(np.abs(b[mask]).max(), 1e-300)


@pytest.mark.parametrize("name", golden_names())
def test_shifted_storage_error_vs_fp64(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    steps = int(d["nsteps"])
    _, u64, _, _ = _run(case, "fp64", steps)
    fluid = ~case.solid
    _, u32, _, _ = _run(case, "fp32_shifted", steps)
    _, u16, _, _ = _run(case, "fp16_shifted", steps)
    assert _rel(u32, u64, fluid) <= FP32_U_TOL
    assert _rel(u16, u64, fluid) <= FP16_U_TOL


# (kind, nodes per thread, threads per block, stages): every autotuner candidate
# kind 2: node pairs from shared-memory tiles of 2048 bytes per plane row
_TILES = {"fp32_shifted": [(2, 2, 128, 2), (2, 2, 128, 3), (2, 2, 256, 2), (2, 2, 64, 2)],
          "fp16_shifted": [(2, 2, 256, 2), (2, 2, 256, 3), (2, 2, 512, 2), (2, 2, 128, 2)]}
_SCALAR = [(0, 1, 128, 0), (0, 1, 256, 0), (0, 1, 128, 1), (0, 1, 256, 1), (0, 1, 128, 2),
           (0, 1, 256, 2)]
_PAIRS = [(3, 2, 128, 0), (3, 2, 256, 0), (3, 2, 128, 1), (3, 2, 256, 2), (3, 2, 128, 3)]
SHIFTED_VARIANTS = {
    "fp32_shifted": _TILES["fp32_shifted"] + _SCALAR + _PAIRS,
    "fp16_shifted": _TILES["fp16_shifted"] + _SCALAR + _PAIRS,
}


@pytest.mark.parametrize("storage,variants", [
    ("fp64", [(0, 1, 128, 0), (0, 1, 256, 0), (0, 1, 512, 0)]),
    ("fp32_shifted", SHIFTED_VARIANTS["fp32_shifted"]),
    ("fp16_shifted", SHIFTED_VARIANTS["fp16_shifted"])])
def test_every_launch_shape_agrees(storage, variants):
    """The autotuner may pick any candidate: all must give the same result
    (FP64 bit for bit; shifted storage within one rounding per step)."""
    case_d, _ = load_golden("channel_cylinder_abb")
    case = Case(case_d)
    outs = [_run(case, storage, 40, v) for v in variants]
    for (r, u, p, shape), v in zip(outs, variants):
        assert shape == v
    r0, u0, p0, _ = outs[0]
    fluid = ~case.solid
    for r, u, p, _ in outs[1:]:
        if storage == "fp64":
            assert np.array_equal(u, u0) and np.array_equal(p, p0)
        else:
            assert _rel(u, u0, fluid) <= 1e-5


def test_mrt_fp64_matches_oracle():
    from oracle.setup import build_state
    from oracle import lbm_np
    case_d, _ = load_golden("poiseuille_guo2")
    case_d["collision_dict"]["fluid"]["model"] = "MRT"
    case_d["collision_dict"]["fluid"]["mrt_rates"] = {"s_e": 1.4, "s_eps": 1.4, "s_q": 1.2}
    st = build_state(case_d)
    lbm_np.run(st, 300)
    case = Case(case_d)
    rho, u, pop, _ = _run(case, "fp64", 300)
    ref_u = st.inner(st.velocity)
    ref_r = st.inner(st.density)
    assert np.abs(rho - ref_r).max() <= MRT_ATOL
    assert np.abs(u - ref_u).max() <= MRT_ATOL
    assert np.abs(u - ref_u).max() <= 1e-10 * np.abs(ref_u).max()


def test_mrt_with_all_rates_omega_is_bgk():
    """M^-1 S M = omega I: MRT with every rate = omega reduces to BGK."""
    case_d, _ = load_golden("poiseuille_guo2")
    case = Case(case_d)
    _, u_bgk, _, _ = _run(case, "fp64", 200)
    om = case.omega
    case_d["collision_dict"]["fluid"]["model"] = "MRT"
    case_d["collision_dict"]["fluid"]["mrt_rates"] = {"s_e": om, "s_eps": om, "s_q": om, "s_nu": om}
    case_m = Case(case_d)
    _, u_mrt, _, _ = _run(case_m, "fp64", 200)
    assert np.abs(u_mrt - u_bgk).max() <= MRT_ATOL


def test_cavity_128_20000_steps_bit_exact_vs_c_oracle():
    """Lid-driven cavity 128x128, Re 100, 20,000 steps (the full cavity run)."""
    from oracle.setup import build_state
    from oracle.clib import COracle
    case_d = workloads.cavity(128)
    st = build_state(case_d)
    co = COracle(st)
    co.initialize()
    co.run(20000)
    case = Case(case_d)
    rho, u, pop, _ = _run(case, "fp64", 20000)
    assert np.array_equal(rho, st.inner(st.density))
    assert np.array_equal(u, st.inner(st.velocity))
    # FP32 shifted against the same FP64 field
    _, u32, _, _ = _run(case, "fp32_shifted", 20000)
    assert _rel(u32, u, np.ones_like(case.solid)) <= FP32_U_TOL


def test_cylinder_small_bit_exact_vs_c_oracle():
    """Cylinder channel (anti-bounce-back inlet/outlet) at 512x128, 300 steps."""
    from oracle.setup import build_state
    from oracle.clib import COracle
    case_d = workloads.cylinder(nx=512, ny=128, radius=16.0, center=(128, 67))
    st = build_state(case_d)
    co = COracle(st)
    co.initialize()
    co.run(300)
    case = Case(case_d)
    rho, u, _, _ = _run(case, "fp64", 300)
    m = ~case.solid
    assert np.array_equal(rho[m], st.inner(st.density)[m])
    assert np.array_equal(u[m], st.inner(st.velocity)[m])


def test_poiseuille_mrt_guo_full_size_vs_analytic():
    """1024x512 MRT + Guo, 50,000 steps: FP64 and FP32 against the analytic
    start-up profile and FP32 against FP64."""
    case_d, par = workloads.poiseuille()
    case = Case(case_d)
    steps = 50000
    _, u64, _, _ = _run(case, "fp64", steps)
    _, u32, _, _ = _run(case, "fp32_shifted", steps)
    prof = workloads.poiseuille_startup_profile(case.ny, par["gx"], par["kin_visc"], steps)
    ux64 = u64[:, :, 0]
    # x-uniform flow
    assert np.abs(ux64 - ux64[:1]).max() <= 1e-12 * np.abs(ux64).max()
    # against the start-up profile: measured 4.3e-6 (FP64) and 3.8e-6 (FP32)
    err = np.abs(ux64[0] - prof).max() / prof.max()
    assert err < 1e-5, err
    err32 = np.abs(u32[:, :, 0] - prof[None, :]).max() / prof.max()
    assert err32 < 1e-5, err32
    assert _rel(u32, u64, np.ones(u64.shape, bool)) <= FP32_STARTUP_TOL


# FP32 conserves what its populations hold: long runs stay at the 1e-7 level
FP32_LONG_TOL = 1e-6
FP32_MASS_DRIFT = 1e-10


def test_fp32_closed_cavity_conserves_mass():
    """Closed 256^2 cavity, 10,000 steps: relative change of the total mass
    (the lid moves tangentially, so the exact mass is constant)."""
    from pylabolt_gb300 import workloads
    case = Case(workloads.cavity(256, re=100.0, lid=0.01))
    with FluidLBM(case, storage="fp32_shifted") as s:
        s.initialize()
        s.step(1)
        m0 = s.conservation()[0]
        s.step(9999)
        m1 = s.conservation()[0]
    assert abs(m1 - m0) / m0 <= FP32_MASS_DRIFT


@pytest.mark.parametrize("coll", ["BGK", "MRT"])
def test_fp32_long_run_against_fp64(coll):
    """1024x256 channel with a cylinder, pressure inlet / outlet, 5000 steps:
    FP32-shifted velocity against FP64 (relative L2 over fluid nodes).  A
    collision whose FP32 rounding does not conserve mass and momentum drifts
    linearly in time and fails this (it measured 1e-5-scale errors)."""
    from pylabolt_gb300 import workloads
    case = Case(workloads.cylinder(nx=1024, ny=256, radius=16.0, center=(256, 131), model=coll,
                                   seed=5))
    fluid = ~case.solid
    _, u64, _, _ = _run(case, "fp64", 5000)
    _, u32, _, _ = _run(case, "fp32_shifted", 5000)
    assert np.linalg.norm(u32[fluid] - u64[fluid]) / np.linalg.norm(u64[fluid]) <= FP32_LONG_TOL


def test_fp32_mrt_poiseuille_long_run():
    """Gravity-driven Poiseuille, MRT + Guo 2nd order, 20,000 steps."""
    from pylabolt_gb300 import workloads
    case_d, _ = workloads.poiseuille(nx=64, ny=128)
    case = Case(case_d)
    fluid = ~case.solid
    _, u64, _, _ = _run(case, "fp64", 20000)
    _, u32, _, _ = _run(case, "fp32_shifted", 20000)
    assert np.linalg.norm(u32[fluid] - u64[fluid]) / np.linalg.norm(u64[fluid]) <= FP32_LONG_TOL


@pytest.mark.parametrize("storage", ["fp32_shifted", "fp16_shifted"])
@pytest.mark.parametrize("coll", ["BGK", "MRT"])
def test_node_pairs_match_the_scalar_kernel(storage, coll):
    """The node-pair kernel on a grid wide enough for its two-node fast path
    (whole bulk segments), with moment and residual steps: the same fields
    and residuals as the one-node-per-thread kernel (the per-node arithmetic
    is the same code)."""
    case = Case(workloads.cylinder(nx=512, ny=128, radius=16.0, center=(128, 67), model=coll))
    fluid = ~case.solid
    outs = []
    for v in ((0, 1, 128, 0), (3, 2, 128, 0), (3, 2, 256, 2), (3, 2, 128, 1)) + tuple(_TILES[storage]):
        os.environ["LBM_VARIANT"] = ",".join(str(i) for i in v)
        try:
            with FluidLBM(case, storage=storage) as sim:
                sim.initialize()
                sim.step(57, residual=True)
                r1 = sim.residual()
                sim.step(43, moments=True, residual=True)
                r2 = sim.residual()
                assert sim.kernel_variant == v
                outs.append((sim.moments()[1], sim.populations(), r1, r2))
        finally:
            del os.environ["LBM_VARIANT"]
    u0, p0, a0, b0 = outs[0]
    for u, p, a, b in outs[1:]:
        assert _rel(u, u0, fluid) <= 1e-6
        np.testing.assert_allclose(a, a0, rtol=1e-6)
        np.testing.assert_allclose(b, b0, rtol=1e-6)


@pytest.mark.parametrize("storage", ["fp32_shifted", "fp16_shifted"])
@pytest.mark.parametrize("coll,forcing", [("BGK", None), ("MRT", None), ("BGK", "guo_second_order")])
@pytest.mark.parametrize("shape", [(2048 + 96, 70), (1000, 33)])
def test_tile_kernel_matches_node_pairs(storage, coll, forcing, shape):
    """The node-pair kernel fed by shared-memory tiles runs the node-pair
    arithmetic on the same incoming words: in FP32 the same populations and
    moments bit for bit, on grids that end inside a tile and rows whose tiles
    straddle the cylinder.  The residual sums are FP32 sums in another order
    (other blocks), so they agree to a few FP32 roundings."""
    nx, ny = shape
    cd = workloads.cylinder(nx=nx, ny=ny, radius=9.0, center=(nx // 3, ny // 2 + 1), model=coll)
    if forcing:
        cd["collision_dict"]["fluid"]["forcing_model"] = forcing
        cd["forcing_dict"] = {"gravity": [2e-6, 0.0]}
    case = Case(cd)
    outs = []
    for v in [(3, 2, 128, 1)] + _TILES[storage]:
        os.environ["LBM_VARIANT"] = ",".join(str(i) for i in v)
        try:
            with FluidLBM(case, storage=storage) as sim:
                sim.initialize()
                sim.step(31, residual=True)
                r1 = sim.residual()
                sim.step(20, moments=True, residual=True)
                r2 = sim.residual()
                assert sim.kernel_variant == v
                outs.append((sim.moments(), sim.populations(), r1, r2))
        finally:
            del os.environ["LBM_VARIANT"]
    (rho0, u0), p0, a0, b0 = outs[0]
    fluid = ~case.solid
    for (rho, u), p, a, b in outs[1:]:
        if storage == "fp32_shifted":
            assert np.array_equal(p, p0)
            assert np.array_equal(rho, rho0) and np.array_equal(u, u0)
            np.testing.assert_allclose(a, a0, rtol=1e-6)
            np.testing.assert_allclose(b, b0, rtol=1e-6)
        else:
            # FP16: the two kernels may contract the FP32 arithmetic into
            # FMAs differently, and a last-bit FP32 difference sometimes
            # rounds a stored half the other way; at the small velocities of
            # these 51 steps such flips reach FP16's own accuracy, so the
            # bound is FP16's (a pull or tile error would be of order 1)
            assert _rel(u, u0, fluid) <= 2e-3
            np.testing.assert_allclose(a, a0, rtol=1e-2)
            np.testing.assert_allclose(b, b0, rtol=1e-2)
