"""The zero_gradient boundary on the GPU.

An unknown incoming population i at an edge node b takes pop[b + n - c_i, i]
(n the inward normal; the post-collision value that reaches b + n along i),
or pop[b + n, i] when that source is outside the grid or solid.  The
reference has no kernel of that name, but its single-rank CPU halo exchange
does exactly this on a "periodic" edge (it copies the first inner column into
the ghosts); the zero_gradient fixtures were stepped by the reference that
way (tests/golden/make_golden.py).

* FP64 through the C-ABI is bit-identical to the NumPy oracle after every
  step of the fixture cases, and to the C oracle on a larger channel whose
  outlet is zero_gradient and whose inlet is anti-bounce-back;
* FP32 shifted storage stays within 1e-5 (max |du| / max |u|) of FP64."""
import numpy as np
import pytest

from _golden import golden_names, load_golden
from pylabolt_gb300 import capi, workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

ZG_CASES = [n for n in golden_names() if n.startswith("zero_gradient")]
RES_RTOL = 1e-12
FP32_U_TOL = 1e-5     # max |u32 - u64| / max |u64|


def test_fixtures_exist():
    assert len(ZG_CASES) >= 2


@pytest.mark.parametrize("name", ZG_CASES)
def test_fp64_every_step_vs_numpy_oracle(name):
    from oracle.setup import build_state
    from oracle import lbm_np
    case_d, d = load_golden(name)
    st = build_state(case_d)
    lbm_np.initialize(st)
    res_o = lbm_np.Residue(st)
    case = Case(case_d)
    m = st.fluid
    with FluidLBM(case, storage="fp64") as sim:
        sim.initialize()
        for t in range(1, int(d["nsteps"]) + 1):
            lbm_np.step(st)
            ro = res_o.compute(st)
            sim.step(1, moments=True, residual=True)
            rg = sim.residual()
            rho, u = sim.moments(layout=capi.LAYOUT_PADDED)
            assert np.array_equal(rho[m], st.density[m]), t
            assert np.array_equal(u[m], st.velocity[m]), t
            assert np.array_equal(sim.populations()[m], st.pop[m]), t
            np.testing.assert_allclose(rg, ro, rtol=RES_RTOL, atol=0)


@pytest.mark.parametrize("outlet_last", [False, True])
def test_fp64_channel_outlet_bit_exact_vs_c_oracle(outlet_last):
    from oracle.setup import build_state
    from oracle.clib import COracle
    case_d = workloads.outlet_channel(384, 96, outlet_last)
    st = build_state(case_d)
    co = COracle(st)
    co.initialize()
    case = Case(case_d)
    m = ~case.solid
    with FluidLBM(case, storage="fp64") as sim:
        sim.initialize()
        for n in (1, 49, 250):
            co.run(n)
            sim.step(n, moments=True)
            rho, u = sim.moments()
            assert np.array_equal(rho[m], st.inner(st.density)[m]), n
            assert np.array_equal(u[m], st.inner(st.velocity)[m]), n


@pytest.mark.parametrize("name", ZG_CASES + ["outlet_channel"])
def test_fp32_shifted_within_tolerance_of_fp64(name):
    if name == "outlet_channel":
        case, steps = Case(workloads.outlet_channel(384, 96, True)), 1000
    else:
        case_d, d = load_golden(name)
        case, steps = Case(case_d), int(d["nsteps"])
    us = {}
    for storage in ("fp64", "fp32_shifted"):
        with FluidLBM(case, storage=storage) as sim:
            sim.initialize()
            sim.step(steps, moments=True)
            us[storage] = sim.moments()[1]
    fluid = ~case.solid
    err = (np.abs(us["fp32_shifted"][fluid] - us["fp64"][fluid]).max() /
           np.abs(us["fp64"][fluid]).max())
    assert err <= FP32_U_TOL, err
