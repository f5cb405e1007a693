"""The product's link table and fused-step plan, emulated on the CPU, against
the reference fixtures (bit-exact).  This pins pylabolt_gb300.config and
pylabolt_gb300.geometry without a GPU."""
import numpy as np
import pytest

from _fused_emulator import FusedEmulator
from _golden import golden_names, load_golden
from pylabolt_gb300.config import Case


@pytest.mark.parametrize("name", golden_names())
def test_fused_plan_bit_exact(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    em = FusedEmulator(case)
    assert np.array_equal(em.padded(case.density.ravel()), d["rho0"])
    assert np.array_equal(em.padded(case.velocity.reshape(-1, 2)), d["u0"])
    assert np.array_equal(em.padded(case.solid.ravel()), d["solid"])
    em.initialize()
    nxp, nyp = case.nx + 2, case.ny + 2
    inner = np.zeros((nxp, nyp), dtype=bool)
    inner[1:-1, 1:-1] = True
    m = inner.ravel() & ~d["solid"]
    cps = set(d["checkpoints"].tolist())
    for t in range(1, int(d["nsteps"]) + 1):
        em.step()
        if t in cps:
            assert np.array_equal(em.padded(em.rho)[m], d[f"density_t{t}"][m])
            assert np.array_equal(em.padded(em.u)[m], d[f"velocity_t{t}"][m])
            assert np.array_equal(em.padded(em.fstar)[m], d[f"pop_t{t}"][m])


@pytest.mark.parametrize("outlet_last", [False, True])
def test_fused_plan_zero_gradient_outlet_vs_oracle(outlet_last):
    """A zero_gradient outlet listed before and after the walls (after them,
    its corner sources leave the grid and fall back to pop[b + n, i])."""
    from oracle.setup import build_state
    from oracle import lbm_np
    from pylabolt_gb300 import workloads
    case_d = workloads.outlet_channel(40, 16, outlet_last)
    case = Case(case_d)
    st = build_state(case_d)
    lbm_np.initialize(st)
    em = FusedEmulator(case)
    em.initialize()
    m = st.fluid
    for t in range(1, 41):
        em.step()
        lbm_np.step(st)
        if t in (1, 2, 20, 40):
            assert np.array_equal(em.padded(em.rho)[m], st.density[m]), t
            assert np.array_equal(em.padded(em.u)[m], st.velocity[m]), t
            assert np.array_equal(em.padded(em.fstar)[m], st.pop[m]), t
