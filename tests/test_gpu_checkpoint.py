"""Checkpoint / restart (lbm_save_state / lbm_load_state and the Solver's
checkpoint_interval): a run saved at step 20 and continued in a fresh handle
matches the uninterrupted run bit for bit -- fields, populations, residuals
(the residual history travels with the state) -- for FP64 and FP32-shifted
storage and both population layouts; mismatched cases are refused."""
import os

import numpy as np
import pytest

from _golden import load_golden
from test_moving_cpu import disk_case
from pylabolt_gb300 import capi, output, solver, workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu


def _steps(sim, res):
    sim.step(7, residual=True)
    res.append(sim.residual())
    sim.step(13, moments=True, residual=True)
    res.append(sim.residual())


@pytest.mark.parametrize("storage,layout", [("fp64", "ab"), ("fp32_shifted", "ab"),
                                            ("fp64", "aa"), ("fp32_shifted", "aa")])
@pytest.mark.parametrize("name", ["channel_cylinder_abb", "poiseuille_guo2"])
def test_restart_is_bit_exact(name, storage, layout, monkeypatch):
    # one launch shape for both handles: shapes may round FP32 differently
    monkeypatch.setenv("LBM_VARIANT", "0,1,128,0" if storage == "fp64" else "0,1,128,1")
    case = Case(load_golden(name)[0])
    ra, rb = [], []
    with FluidLBM(case, storage=storage, layout=layout) as a:
        a.initialize()
        _steps(a, ra)                      # t = 20
        state = a.save_state()
        assert a.time == 20
        _steps(a, ra)                      # t = 40
        pa = a.populations()
        ma = a.moments()
    with FluidLBM(case, storage=storage, layout=layout) as b:
        b.initialize()
        b.step(3)                          # whatever it held is replaced
        b.load_state(state)
        assert b.time == 20
        _steps(b, rb)
        assert np.array_equal(b.populations(), pa)
        mb = b.moments()
        assert np.array_equal(ma[0], mb[0]) and np.array_equal(ma[1], mb[1])
    assert np.array_equal(np.array(ra[2:]), np.array(rb))


@pytest.mark.parametrize("storage", ["fp32_shifted", "fp16_shifted"])
def test_restart_keeps_the_tuned_launch_shape(storage, monkeypatch):
    """Without a pinned launch shape each handle runs the autotuner, and
    shapes round FP32 / FP16 differently.  The saved state carries the
    shapes of the saving handle, so a fresh handle continues bit for bit."""
    monkeypatch.delenv("LBM_VARIANT", raising=False)
    monkeypatch.delenv("LBM_TUNE", raising=False)
    case = Case(workloads.cylinder(nx=512, ny=128, radius=16.0, center=(128, 67)))
    ra, rb = [], []
    with FluidLBM(case, storage=storage) as a:
        a.initialize()
        _steps(a, ra)
        state = a.save_state()
        shape = a.kernel_variant
        _steps(a, ra)
        pa = a.populations()
    with FluidLBM(case, storage=storage) as b:
        b.initialize()
        b.load_state(state)
        assert b.kernel_variant == shape
        _steps(b, rb)
        assert np.array_equal(b.populations(), pa)
    assert np.array_equal(np.array(ra[2:]), np.array(rb))


def test_state_of_another_obstacle_layout_or_viscosity_is_refused():
    """Same grid, storage and number of link records, but the cylinder one
    node higher, or another viscosity: the case hash in the state refuses
    both."""
    base = workloads.cylinder(nx=256, ny=64, radius=8.0, center=(64, 35))
    moved = workloads.cylinder(nx=256, ny=64, radius=8.0, center=(64, 36))
    visc = workloads.cylinder(nx=256, ny=64, radius=8.0, center=(64, 35), kin_visc=0.05)
    with FluidLBM(Case(base), storage="fp64") as a:
        a.initialize()
        a.step(5)
        state = a.save_state()
        for other in (moved, visc):
            with FluidLBM(Case(other), storage="fp64") as b:
                b.initialize()
                with pytest.raises(capi.LbmError, match="another"):
                    b.load_state(state)
                b.step(2)
        a.load_state(state)                  # its own state still loads


def test_mismatched_state_is_refused():
    a_case = Case(load_golden("channel_cylinder_abb")[0])
    b_case = Case(load_golden("cavity_lid_first")[0])
    with FluidLBM(a_case, storage="fp64") as a, FluidLBM(b_case, storage="fp64") as b, \
            FluidLBM(a_case, storage="fp32_shifted") as c:
        a.initialize()
        b.initialize()
        c.initialize()
        state = a.save_state()
        for other in (b, c):
            with pytest.raises(capi.LbmError, match="another grid"):
                other.load_state(state)
        bad = state.copy()
        bad[:8] = 0
        with pytest.raises(capi.LbmError, match="not a saved state"):
            a.load_state(bad)
        b.step(2)                            # the refused handles still run
        c.step(2)


def test_solver_resumes_from_checkpoint(tmp_path, monkeypatch, capsys):
    monkeypatch.setattr(output, "package_version", lambda: "0.0.0")
    case = workloads.cavity(64)
    case["control_dict"].update({"end_time": 60, "std_out_interval": 20, "save_interval": 30,
                                 "checkpoint_interval": 20})
    full = tmp_path / "full"
    s = solver.Solver(case, root=str(full), storage="fp64", verbose=False)
    try:
        s.run()
    finally:
        s.close()
    for t in (20, 40, 60):
        assert os.path.exists(full / "output" / "checkpoints" / f"state_t{t}.npy")
    # a second run directory holding the t = 20 checkpoint, started at 20
    part = tmp_path / "part"
    os.makedirs(part / "output" / "checkpoints")
    os.link(full / "output" / "checkpoints" / "state_t20.npy",
            part / "output" / "checkpoints" / "state_t20.npy")
    case["control_dict"]["start_time"] = 20
    s = solver.Solver(case, root=str(part), storage="fp64", verbose=False)
    try:
        s.run()
    finally:
        s.close()
    for t in (30, 60):
        zf = np.load(full / "output" / "fields" / f"t_{t}.npz")
        zp = np.load(part / "output" / "fields" / f"t_{t}.npz")
        for k in zf.files:
            assert np.array_equal(zf[k], zp[k]), (t, k)


@pytest.mark.parametrize("kw", [{"v": (0.05, 0.02), "om": 0.01},
                                {"v": (0.0, 0.0), "om": 0.0, "kind": "calculated", "density": 1.5}])
def test_restart_with_moving_obstacles(kw, monkeypatch):
    """The moving obstacles' device state travels with the step state: the
    restarted run moves them and fills the nodes they leave exactly as the
    uninterrupted one."""
    monkeypatch.setenv("LBM_VARIANT", "0,1,128,0")
    case = Case(disk_case(True, **kw))
    with FluidLBM(case, storage="fp64") as a:
        a.initialize()
        a.step(25, residual=True)
        state = a.save_state()
        a.step(40, moments=True, residual=True)
        ra = a.residual()
        pa, fa, oa = a.populations(), a.node_flags(), a.moving_obstacles()[0]
        ma = a.moments()
    with FluidLBM(case, storage="fp64") as b:
        b.initialize()
        b.load_state(state)
        b.step(40, moments=True, residual=True)
        assert np.array_equal(b.residual(), ra)
        assert np.array_equal(b.populations(), pa)
        assert np.array_equal(b.node_flags(), fa)
        ob = b.moving_obstacles()[0]
        for k in ("center", "velocity", "force"):
            assert np.array_equal(np.asarray(oa[k]), np.asarray(ob[k])), k
        assert oa["omega"] == ob["omega"] and oa["torque"] == ob["torque"]
        mb = b.moments()
        assert np.array_equal(ma[0], mb[0]) and np.array_equal(ma[1], mb[1])
