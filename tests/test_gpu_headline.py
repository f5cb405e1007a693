"""The benchmark's own case at its full size: the 8192 x 2048 channel with a
cylinder of radius 128 (anti-bounce-back inlet / outlet, bounce-back walls
and cylinder, seeded velocity perturbation).

* FP64 storage, with two population buffers and with one updated in place
  (AA), is bit-identical to the C oracle (pinned to the reference's kernels)
  after 12 steps.
* FP32-shifted storage, BGK and MRT, stays within FP32_U_TOL of FP64 (max |du|
  over max |u|) after 1000 steps, the bound the FP32 path is built to."""
import numpy as np
import pytest

from pylabolt_gb300 import workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

FP32_U_TOL = 1e-5


def _velocity(case, storage, steps, layout="ab"):
    with FluidLBM(case, storage=storage, layout=layout) as sim:
        sim.initialize()
        sim.step(steps, moments=True)
        return sim.moments()


def test_cylinder_full_size_fp64_bit_exact_vs_c_oracle():
    from oracle.setup import build_state
    from oracle.clib import COracle
    case_d = workloads.cylinder()
    steps = 12
    st = build_state(case_d)
    co = COracle(st)
    co.initialize()
    co.run(steps)
    case = Case(case_d)
    m = ~case.solid
    for layout in ("ab", "aa"):
        rho, u = _velocity(case, "fp64", steps, layout)
        assert np.array_equal(rho[m], st.inner(st.density)[m]), layout
        assert np.array_equal(u[m], st.inner(st.velocity)[m]), layout


@pytest.mark.parametrize("model", ["BGK", "MRT"])
def test_cylinder_full_size_fp32_error_vs_fp64(model):
    case = Case(workloads.cylinder(model=model))
    steps = 1000
    _, u64 = _velocity(case, "fp64", steps)
    _, u32 = _velocity(case, "fp32_shifted", steps)
    m = ~case.solid
    err = np.abs(u32[m] - u64[m]).max() / np.abs(u64[m]).max()
    assert err <= FP32_U_TOL, err
