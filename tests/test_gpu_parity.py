"""CUDA path (through the C-ABI) against the oracle.

FP64 mode must be bit-identical to the reference-kernel fixtures and to the C
oracle; residuals agree to 1e-12 relative (the reduction order differs)."""
import numpy as np
import pytest

from _golden import golden_names, load_golden
from pylabolt_gb300 import capi
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

RES_RTOL = 1e-12


def _inner_mask(nx, ny, solid_padded):
    m = np.zeros((nx + 2, ny + 2), dtype=bool)
    m[1:-1, 1:-1] = True
    return m.ravel() & ~solid_padded


@pytest.mark.parametrize("name", golden_names())
def test_fp64_bit_exact_vs_reference_fixtures(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    with FluidLBM(case, storage="fp64") as sim:
        sim.initialize()
        m = _inner_mask(case.nx, case.ny, d["solid"])
        cps = set(d["checkpoints"].tolist())
        res = []
        for t in range(1, int(d["nsteps"]) + 1):
            sim.step(1, moments=t in cps, residual=True)
            res.append(sim.residual())
            if t in cps:
                rho, u = sim.moments(layout=capi.LAYOUT_PADDED)
                pop = sim.populations()
                assert np.array_equal(rho[m], d[f"density_t{t}"][m]), t
                assert np.array_equal(u[m], d[f"velocity_t{t}"][m]), t
                assert np.array_equal(pop[m], d[f"pop_t{t}"][m]), t
                # solid nodes keep the body's density / velocity
                s = d["solid"]
                assert np.array_equal(rho[s], d[f"density_t{t}"][s])
        g = d["residuals"][:, 1:]
        np.testing.assert_allclose(np.array(res), g, rtol=RES_RTOL, atol=0)
        assert sim.time == int(d["nsteps"])


def test_graph_replay_equals_single_steps():
    """A long lbm_step (graph-replayed chunks) gives the same bits as one call
    per step."""
    case = Case(load_golden("periodic_moving_disk")[0])
    with FluidLBM(case, storage="fp64") as a, FluidLBM(case, storage="fp64") as b:
        a.initialize()
        b.initialize()
        a.step(101, moments=True)
        for _ in range(100):
            b.step(1)
        b.step(1, moments=True)
        assert np.array_equal(a.populations(), b.populations())
        ra, ua = a.moments()
        rb, ub = b.moments()
        assert np.array_equal(ra, rb) and np.array_equal(ua, ub)
        assert a.kernel_launches == 101


@pytest.mark.parametrize("storage,layout,shape", [("fp64", "ab", "0,1,128,0"),
                                                  ("fp32_shifted", "ab", "3,2,128,1"),
                                                  ("fp32_shifted", "aa", "3,2,128,1")])
def test_step_calls_of_any_length_give_the_same_bits(storage, layout, shape, monkeypatch):
    """Calls of any length -- graph chunks, one graph of the remainder from
    either buffer parity, single steps -- give the bits of one call per step
    (one launch shape for both handles)."""
    monkeypatch.setenv("LBM_VARIANT", shape)
    case = Case(load_golden("channel_cylinder_abb")[0])
    groups = [1, 2, 3, 7, 31, 33, 64, 5, 40, 2]
    with FluidLBM(case, storage=storage, layout=layout) as a, \
            FluidLBM(case, storage=storage, layout=layout) as b:
        a.initialize()
        b.initialize()
        for n in groups:
            a.step(n)
        a.time_steps(21)
        for _ in range(sum(groups) + 21):
            b.step(1)
        a.step(1, moments=True)
        b.step(1, moments=True)
        assert a.time == b.time == sum(groups) + 22
        assert a.kernel_launches == b.kernel_launches
        assert np.array_equal(a.populations(), b.populations())
        assert np.array_equal(a.moments()[1], b.moments()[1])


def test_restart_from_populations_is_bit_exact():
    """set_populations(pop_new) restarts a run: the reference's pop_fluid_new
    after step t, fed back, continues identically."""
    from oracle.setup import build_state
    from oracle import lbm_np
    case_d, _ = load_golden("channel_cylinder_abb")
    st = build_state(case_d)
    lbm_np.run(st, 10)
    pop_new = st.pop_new.copy()
    pop_new[~st.fluid] = 0.0
    for _ in range(15):
        lbm_np.step(st)
    case = Case(case_d)
    with FluidLBM(case, storage="fp64") as sim:
        sim.initialize()
        sim.set_populations(pop_new)
        sim.step(15, moments=True)
        rho, u = sim.moments(layout=capi.LAYOUT_PADDED)
        m = st.fluid
        assert np.array_equal(rho[m], st.density[m])
        assert np.array_equal(u[m], st.velocity[m])
        assert np.array_equal(sim.populations()[m], st.pop[m])
