"""AA (in-place) population layout on the GPU.

FP64 storage must reproduce the reference-kernel fixtures bit for bit, like
the two-buffer layout, after even and odd step counts (populations read back
through both phases' addressing); residuals, forces and conservation sums
agree with the two-buffer run; FP32 / FP16 shifted storage agrees with the
two-buffer run within AB_TOL (the same node arithmetic in a different
kernel)."""
import numpy as np
import pytest

from _golden import golden_names, load_golden
from pylabolt_gb300 import capi, workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

RES_RTOL = 1e-12
FORCE_RTOL = 1e-12
# max |u_aa - u_ab| / max |u_ab|.  Kernels may contract the collision's FP32
# arithmetic into FMAs differently; in FP16 storage an occasional flipped
# rounding of a stored half then follows, and over 501 steps these add up to
# about FP16's own error against FP64 (8e-4 here), so FP16 is bounded at
# 2e-3: a layout error would be of order 1.
AB_TOL = {"fp32_shifted": 1e-6, "fp16_shifted": 2e-3}


def _inner_mask(nx, ny, solid_padded):
    m = np.zeros((nx + 2, ny + 2), dtype=bool)
    m[1:-1, 1:-1] = True
    return m.ravel() & ~solid_padded


@pytest.mark.parametrize("name", golden_names(zero_gradient=False))
def test_aa_fp64_bit_exact_vs_reference_fixtures(name):
    case_d, d = load_golden(name)
    case = Case(case_d)
    with FluidLBM(case, storage="fp64", layout="aa") as sim:
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
        np.testing.assert_allclose(np.array(res), d["residuals"][:, 1:], rtol=RES_RTOL, atol=0)


@pytest.mark.parametrize("name", golden_names(zero_gradient=False))
def test_aa_forces_and_conservation_match_two_buffers(name):
    case = Case(load_golden(name)[0])
    with FluidLBM(case, storage="fp64") as ab, FluidLBM(case, storage="fp64", layout="aa") as aa:
        ab.initialize()
        aa.initialize()
        for n in (0, 1, 1, 2, 5):   # forces read p_t and the next step's links in both phases
            if n:
                ab.step(n)
                aa.step(n)
            fa, fb = aa.forces(), ab.forces()
            np.testing.assert_allclose(fa["obstacles"], fb["obstacles"], rtol=FORCE_RTOL, atol=1e-15)
            np.testing.assert_allclose(fa["walls"], fb["walls"], rtol=FORCE_RTOL, atol=1e-15)
            np.testing.assert_allclose(aa.conservation(), ab.conservation(), rtol=1e-13, atol=1e-13)
            assert np.array_equal(aa.populations(), ab.populations())


def test_aa_graph_replay_and_restart():
    """Graph-replayed chunks (odd and even starting phase) equal single steps;
    set_populations restarts from an even phase."""
    case = Case(load_golden("periodic_moving_disk")[0])
    with FluidLBM(case, storage="fp64", layout="aa") as a, \
            FluidLBM(case, storage="fp64", layout="aa") as b, \
            FluidLBM(case, storage="fp64") as c:
        for s in (a, b, c):
            s.initialize()
        a.step(1)
        a.step(100, moments=True)      # graphs start on an odd phase
        for _ in range(101):
            b.step(1)
        c.step(101)
        pa = a.populations()
        assert np.array_equal(pa, b.populations())
        assert np.array_equal(pa, c.populations())
        a.step(64)
        c.step(64)
        assert np.array_equal(a.populations(), c.populations())
        pop = c.populations()
        b.set_populations(pop)
        c.set_populations(pop)
        b.step(33, moments=True)
        c.step(33, moments=True)
        assert np.array_equal(b.populations(), c.populations())
        rb, ub = b.moments()
        rc, uc = c.moments()
        assert np.array_equal(rb, rc) and np.array_equal(ub, uc)


@pytest.mark.parametrize("storage", ["fp32_shifted", "fp16_shifted"])
@pytest.mark.parametrize("coll", ["BGK", "MRT"])
def test_aa_shifted_storage_matches_two_buffers(storage, coll, monkeypatch):
    """Both layouts on the node-pair kernel (the AA default for shifted
    storage), 501 steps."""
    monkeypatch.setenv("LBM_VARIANT", "3,2,128,1")
    case = Case(workloads.cylinder(nx=512, ny=128, radius=16.0, center=(128, 67), model=coll))
    out = {}
    for layout in ("ab", "aa"):
        with FluidLBM(case, storage=storage, layout=layout) as sim:
            sim.initialize()
            sim.step(501, moments=True)
            out[layout] = sim.moments()[1]
            if layout == "aa":
                assert sim.device_bytes < out["bytes_ab"]
            else:
                out["bytes_ab"] = sim.device_bytes
    err = np.abs(out["aa"] - out["ab"]).max() / np.abs(out["ab"]).max()
    assert err <= AB_TOL[storage], err


def test_aa_rejections_on_handle():
    case = Case(load_golden("channel_cylinder_abb")[0])
    with FluidLBM(case, storage="fp64", layout="aa") as sim:
        sim.initialize()
        with pytest.raises(capi.LbmError, match="AA population layout"):
            sim.adjoint_forward(4, 2)


def test_device_bytes_accounting():
    """The residual's previous-step fields are allocated by the first residual
    step; freed and re-made workspaces (staging, adjoint plans) are counted
    once."""
    case = Case(load_golden("cavity_lid_first")[0])
    with FluidLBM(case, storage="fp32_shifted") as sim:
        sim.initialize()
        b0 = sim.device_bytes
        sim.step(2)
        assert sim.device_bytes == b0
        sim.step(1, residual=True)
        b1 = sim.device_bytes
        assert b1 > b0
        sim.step(3, residual=True)
        sim.populations()
        b2 = sim.device_bytes
        sim.populations()
        assert sim.device_bytes == b2
        sim.initialize()
        sim.adjoint_forward(10, 2)
        b3 = sim.device_bytes
        sim.initialize()
        sim.adjoint_forward(10, 3)
        sim.initialize()
        sim.adjoint_forward(10, 2)
        assert sim.device_bytes == b3


@pytest.mark.parametrize("which", ["mrt_cylinder", "body_force_channel"])
def test_aa_fp64_matches_two_buffers(which):
    """MRT with Guo forcing and a per-node body-force field through the AA
    phases: FP64 bit for bit against the two-buffer run (odd and even step
    counts, moments and populations)."""
    if which == "mrt_cylinder":
        case_d = workloads.cylinder(nx=256, ny=96, radius=10.0, center=(64, 49), model="MRT")
        case_d["collision_dict"]["fluid"]["forcing_model"] = "guo_second_order"
        case_d["forcing_dict"] = {"gravity": [1e-6, 2e-7]}
    else:
        case_d = workloads.adjoint_channel(nx=192, ny=96)
    case = Case(case_d)
    with FluidLBM(case, storage="fp64") as ab, FluidLBM(case, storage="fp64", layout="aa") as aa:
        ab.initialize()
        aa.initialize()
        for n in (37, 40):
            ab.step(n, moments=True)
            aa.step(n, moments=True)
            ra, ua = aa.moments()
            rb, ub = ab.moments()
            assert np.array_equal(ra, rb) and np.array_equal(ua, ub)
            assert np.array_equal(aa.populations(), ab.populations())


@pytest.mark.parametrize("storage", ["fp32_shifted", "fp16_shifted"])
@pytest.mark.parametrize("coll", ["BGK", "MRT"])
def test_aa_node_pairs_match_scalar_aa(storage, coll, monkeypatch):
    """The AA node-pair kernel (two nodes per thread; aligned words in the
    even phase, pulls of word pairs and per-node pushes in the odd phase) on a
    grid wide enough for its fast path, odd and even step counts, with
    moment and residual steps: the same fields and residuals as the
    one-node-per-thread AA kernel, and the two-buffer run within AB_TOL."""
    case = Case(workloads.cylinder(nx=512, ny=128, radius=16.0, center=(128, 67), model=coll))
    fluid = ~case.solid
    outs = []
    for layout, v in (("aa", "0,1,128,1"), ("aa", "3,2,128,1"), ("aa", "3,2,256,0"),
                      ("ab", "0,1,128,1")):
        monkeypatch.setenv("LBM_VARIANT", v)
        with FluidLBM(case, storage=storage, layout=layout) as sim:
            sim.initialize()
            res = []
            for n in (1, 20, 37):
                sim.step(n, moments=True, residual=True)
                res.append(sim.residual())
            want = tuple(int(i) for i in v.split(","))
            assert sim.kernel_variant[:3] == want[:3]
            outs.append((sim.moments()[1], np.array(res)))
    u0, r0 = outs[0]
    for u, r in outs[1:3]:
        assert np.abs(u - u0)[fluid].max() <= 1e-6 * np.abs(u0[fluid]).max()
        np.testing.assert_allclose(r, r0, rtol=1e-5)
    uab = outs[3][0]
    assert np.abs(u0 - uab)[fluid].max() <= AB_TOL[storage] * np.abs(uab[fluid]).max()


def test_aa_default_launch_shape():
    """Without LBM_VARIANT the AA layout runs the scalar kernel for FP64, the
    node-pair kernel for FP32 storage and the node-pair tile kernel (two
    pairs of a 1024-node tile per thread, two stages) for FP16."""
    import os
    assert "LBM_VARIANT" not in os.environ
    case = Case(load_golden("channel_cylinder_abb")[0])
    for storage, shape in (("fp64", (0, 1, 128, 0)), ("fp32_shifted", (3, 2, 128, 1)),
                           ("fp16_shifted", (2, 2, 256, 2))):
        with FluidLBM(case, storage=storage, layout="aa") as sim:
            sim.initialize()
            sim.step(3)
            assert sim.kernel_variant == shape


@pytest.mark.parametrize("storage", ["fp32_shifted", "fp16_shifted"])
@pytest.mark.parametrize("coll,forcing", [("BGK", None), ("MRT", None), ("BGK", "guo_second_order")])
@pytest.mark.parametrize("shape", [(2144, 70), (1000, 33)])
def test_aa_tile_kernel_matches_aa_node_pairs(storage, coll, forcing, shape, monkeypatch):
    """The node-pair tile kernel in the AA layout (the even phase staging a
    tile's own slots, the odd phase the pulled rows, pushes to global memory)
    against the AA node-pair kernel, after even and odd step counts with
    moment and residual steps: FP32 the same populations and moments bit for
    bit, residuals within FP32 summation order; FP16 within AB_TOL.  The grids
    end inside a tile, and their rows are not whole tiles (AA rows are
    padded to 128 bytes)."""
    nx, ny = shape
    cd = workloads.cylinder(nx=nx, ny=ny, radius=9.0, center=(nx // 3, ny // 2 + 1), model=coll)
    if forcing:
        cd["collision_dict"]["fluid"]["forcing_model"] = forcing
        cd["forcing_dict"] = {"gravity": [2e-6, 0.0]}
    case = Case(cd)
    fluid = ~case.solid
    tp = 2048 // (2 if storage == "fp16_shifted" else 4) // 2   # pairs of a tile
    outs = []
    for v in ("3,2,128,1", f"2,2,{tp // 2},2", f"2,2,{tp // 2},3"):
        monkeypatch.setenv("LBM_VARIANT", v)
        with FluidLBM(case, storage=storage, layout="aa") as sim:
            sim.initialize()
            res = []
            for n in (1, 20, 36):
                sim.step(n, moments=True, residual=True)
                res.append(sim.residual())
            assert sim.kernel_variant == tuple(int(i) for i in v.split(","))
            rho, u = sim.moments()
            outs.append((rho, u, sim.populations(), np.array(res)))
    rho0, u0, p0, r0 = outs[0]
    for rho, u, p, r in outs[1:]:
        if storage == "fp32_shifted":
            assert np.array_equal(p, p0)
            assert np.array_equal(rho, rho0) and np.array_equal(u, u0)
            np.testing.assert_allclose(r, r0, rtol=1e-6)
        else:
            assert np.abs(u - u0)[fluid].max() <= AB_TOL[storage] * np.abs(u0[fluid]).max()
