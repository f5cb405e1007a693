"""The oracle against fixtures generated by the reference's own kernels.

The fixtures come from tests/golden/make_golden.py (reference CPU kernels run
as Python).  Both restatements -- NumPy and C -- must reproduce every
checkpoint and the residual history bit for bit."""
import numpy as np
import pytest

from _golden import golden_names, load_golden
from oracle import lbm_np
from oracle.clib import COracle
from oracle.setup import build_state

NAMES = golden_names()


def test_fixtures_present():
    assert len(NAMES) >= 6


def _compare(st, d, t):
    fl = st.fluid
    for key, arr in (("density", st.density), ("velocity", st.velocity),
                     ("pop", st.pop), ("pop_new", st.pop_new)):
        g = d[f"{key}_t{t}"]
        m = fl if key.startswith("pop") else slice(None)
        assert np.array_equal(arr[m], g[m]), f"{key} differs at t={t}"


@pytest.mark.parametrize("name", NAMES)
def test_setup_matches_reference_state(name):
    case, d = load_golden(name)
    st = build_state(case)
    assert np.array_equal(st.density, d["rho0"])
    assert np.array_equal(st.velocity, d["u0"])
    assert np.array_equal(st.solid, d["solid"])


@pytest.mark.parametrize("name", NAMES)
def test_numpy_oracle_bit_exact(name):
    case, d = load_golden(name)
    st = build_state(case)
    lbm_np.initialize(st)
    res = lbm_np.Residue(st)
    cps = set(d["checkpoints"].tolist())
    hist = []
    for t in range(1, int(d["nsteps"]) + 1):
        lbm_np.step(st)
        hist.append(res.compute(st))
        if t in cps:
            _compare(st, d, t)
    assert np.array_equal(np.array(hist), d["residuals"][:, 1:])


@pytest.mark.parametrize("name", NAMES)
def test_c_oracle_bit_exact(name):
    case, d = load_golden(name)
    st = build_state(case)
    co = COracle(st)
    co.initialize()
    cps = set(d["checkpoints"].tolist())
    hist = []
    for t in range(1, int(d["nsteps"]) + 1):
        co.run(1)
        hist.append(co.residue())
        if t in cps:
            _compare(st, d, t)
    assert np.array_equal(np.array(hist), d["residuals"][:, 1:])


def test_lattice_constants_match_reference_values():
    """pylabolt/base/lattice.py:41-60 (and tests/unit/test_lattice.py:94-135)."""
    from oracle.setup import CX, CY, W, INV, INV_CS_2, INV_CS_4
    assert list(CX) == [0, 1, 0, -1, 0, 1, -1, -1, 1]
    assert list(CY) == [0, 0, 1, 0, -1, 1, 1, -1, -1]
    assert list(INV) == [0, 3, 4, 1, 2, 7, 8, 5, 6]
    assert np.all(W == np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36]))
    assert INV_CS_2 == 2.999999999999999 and INV_CS_4 == 8.999999999999995


def test_selfcopy_equals_wrap_for_x_uniform_flow():
    """The single-rank CPU halo (self copy) and the GPU wrap agree when the
    flow does not vary in x (Poiseuille)."""
    case, _ = load_golden("poiseuille_guo2")
    a = build_state(case, periodic_mode="wrap")
    b = build_state(case, periodic_mode="selfcopy")
    lbm_np.run(a, 40)
    lbm_np.run(b, 40)
    assert np.array_equal(a.pop_new[a.fluid], b.pop_new[b.fluid])


@pytest.mark.parametrize("name", [n for n in NAMES if n.startswith("zero_gradient")])
def test_zero_gradient_is_the_reference_cpu_self_copy(name):
    """The zero_gradient fixtures were stepped by the reference with periodic
    edges and its single-rank CPU halo exchange (a copy of the first inner
    column / row into the ghosts).  The oracle run on those very
    dictionaries in its self-copy mode, and on the zero_gradient twin, give
    the fixture bit for bit: the two definitions are one."""
    import json
    case_zg, d = load_golden(name)
    ref_case = json.loads(str(d["ref_case_json"]))
    for region, rd in ref_case["initial_fields_dict"].items():
        for fname, spec in rd["fluid"].items():
            if spec["type"] == "array":
                spec["value"] = d[f"init_{region}_{fname}"]
    assert str(d["halo"]) == "selfcopy"
    a = build_state(ref_case, periodic_mode="selfcopy")
    b = build_state(case_zg)
    assert a.x_periodic or a.y_periodic
    assert not (b.x_periodic or b.y_periodic)
    nsteps = int(d["nsteps"])
    lbm_np.run(a, nsteps)
    lbm_np.run(b, nsteps)
    _compare(a, d, nsteps)
    _compare(b, d, nsteps)
