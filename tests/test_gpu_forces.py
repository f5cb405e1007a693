"""Momentum-exchange forces on the GPU (lbm_forces) against the reference's
force kernels on the golden populations and against the oracle on a larger
channel.  FP64 storage: the per-link values are bit-exact, the sums agree to
1e-12 relative (their order differs); FP32 storage within FORCE_FP32_RTOL of
the FP64 forces."""
import numpy as np
import pytest

from _golden import golden_names, load_golden
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-12
FORCE_FP32_RTOL = 1e-4   # relative to the largest force component of the case


def _check(got, d, t):
    np.testing.assert_allclose(got["obstacles"], d[f"force_obstacles_t{t}"],
                               rtol=FORCE_RTOL, atol=1e-15)
    np.testing.assert_allclose(got["walls"], d[f"force_walls_t{t}"], rtol=FORCE_RTOL, atol=1e-15)


@pytest.mark.parametrize("name", golden_names())
def test_forces_fp64_against_reference_kernels(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    with FluidLBM(case, storage="fp64") as sim:
        sim.initialize()
        assert sim.force_names == (d["obstacle_names"].tolist(), d["wall_names"].tolist())
        _check(sim.forces(), d, 0)
        t = 0
        for cp in sorted(d["checkpoints"].tolist()):
            sim.step(cp - t)
            t = cp
            _check(sim.forces(), d, t)


@pytest.mark.parametrize("name", ["channel_cylinder_abb", "cavity_lid_last"])
def test_forces_fp32_close_to_fp64(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    t = int(d["nsteps"])
    with FluidLBM(case, storage="fp32_shifted") as sim:
        sim.initialize()
        sim.step(t)
        got = sim.forces()
    ref_o, ref_w = d[f"force_obstacles_t{t}"], d[f"force_walls_t{t}"]
    scale = max(np.abs(ref_o).max(initial=0), np.abs(ref_w).max(initial=0))
    assert np.abs(got["obstacles"] - ref_o).max(initial=0) <= FORCE_FP32_RTOL * scale
    assert np.abs(got["walls"] - ref_w).max(initial=0) <= FORCE_FP32_RTOL * scale


def test_cylinder_channel_forces_against_oracle():
    """256x64 channel, anti-bounce-back inlet/outlet, cylinder r = 8, 300
    steps: drag, lift and torque of the cylinder and the wall forces against
    the oracle's restatement of the reference force kernels on the C oracle's
    pop / pop_new."""
    from oracle.clib import COracle
    from oracle.setup import build_state
    from oracle import lbm_np
    from pylabolt_gb300 import workloads
    from pylabolt_gb300.obstacles import Geometry
    case_d = workloads.cylinder(nx=256, ny=64, radius=8.0, center=(64, 35), kin_visc=0.02,
                                rho_in=1.001, seed=3, amp=1e-4)
    nsteps = 300
    st = build_state(case_d)
    co = COracle(st)
    co.initialize()
    co.run(nsteps)
    case = Case(case_d)
    geo = Geometry(case)
    npad = (case.nx + 2) * (case.ny + 2)
    solid, sid, fb = (geo.solid.reshape(npad), geo.solid_id.reshape(npad),
                      geo.fluid_boundary.reshape(npad))
    o = case.obstacles[0]
    ref_cyl = lbm_np.obstacle_force_torque(st.pop, st.pop_new, solid, sid, fb, case.nx, case.ny,
                                           o.center, o.id, case.x_periodic, case.y_periodic)
    walls = [el for el in case.elements if el.wall]
    ref_w = [lbm_np.boundary_force(st.pop, st.pop_new, solid,
                                   (el.xs + 1) * (case.ny + 2) + el.ys + 1, el.out_list, el.inv_list)
             for el in walls]
    with FluidLBM(case, storage="fp64") as sim:
        sim.initialize()
        sim.step(nsteps)
        got = sim.forces()
    np.testing.assert_allclose(got["obstacles"][0], ref_cyl, rtol=FORCE_RTOL, atol=1e-14)
    np.testing.assert_allclose(got["walls"], np.array(ref_w), rtol=FORCE_RTOL, atol=1e-14)


def test_ellipse_channel_against_c_oracle():
    """512x128 channel with an ellipse (semi-axes 24 and 8, inclined 20
    degrees) and anti-bounce-back inlet / outlet, 300 steps: FP64 fields bit
    for bit against the C oracle, the ellipse's force and torque against the
    oracle's restatement of the reference force kernel, FP32 shifted within
    1e-5 of FP64."""
    from oracle.clib import COracle
    from oracle.setup import build_state
    from oracle import lbm_np
    from pylabolt_gb300 import workloads
    from pylabolt_gb300.obstacles import Geometry
    case_d = workloads.ellipse_channel(512, 128)
    nsteps = 300
    st = build_state(case_d)
    co = COracle(st)
    co.initialize()
    co.run(nsteps)
    case = Case(case_d)
    assert case.solid.sum() > 0 and np.array_equal(case.solid, st.inner(st.solid))
    geo = Geometry(case)
    npad = (case.nx + 2) * (case.ny + 2)
    o = case.obstacles[0]
    ref = lbm_np.obstacle_force_torque(st.pop, st.pop_new, geo.solid.reshape(npad),
                                       geo.solid_id.reshape(npad), geo.fluid_boundary.reshape(npad),
                                       case.nx, case.ny, o.center, o.id, case.x_periodic,
                                       case.y_periodic)
    us = {}
    for storage in ("fp64", "fp32_shifted"):
        with FluidLBM(case, storage=storage) as sim:
            sim.initialize()
            sim.step(nsteps, moments=True)
            rho, us[storage] = sim.moments()
            if storage == "fp64":
                m = ~case.solid
                assert np.array_equal(rho[m], st.inner(st.density)[m])
                assert np.array_equal(us[storage][m], st.inner(st.velocity)[m])
                # the torque (4e-4) is a sum of ~10^3 arm x momentum terms of
                # either sign, summed in another order on the GPU: 1e-13 absolute
                np.testing.assert_allclose(sim.forces()["obstacles"][0], ref, rtol=FORCE_RTOL,
                                           atol=1e-13)
    m = ~case.solid
    err = np.abs(us["fp32_shifted"][m] - us["fp64"][m]).max() / np.abs(us["fp64"][m]).max()
    assert err <= 1e-5, err
