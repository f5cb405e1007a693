"""Failure detection on the GPU, with the failure made on the host: a NaN or an
infinity seeded into the initial density of a 16x16 cavity makes the fused
residual pass count non-finite nodes, and lbm_residual returns
LBM_ERR_NONFINITE with the count.  Nothing faults: the handle stays usable and
a re-initialised run reports a finite residual again."""
import re

import numpy as np
import pytest

from pylabolt_gb300 import capi, workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["fp64", "fp32_shifted", "fp16_shifted"])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
@pytest.mark.parametrize("layout", ["ab", "aa"])
def test_nonfinite_density_is_reported(storage, bad, layout):
    case = Case(workloads.cavity(16))
    rho = case.density.copy()
    rho[5, 7] = bad
    rho[9, 2] = bad
    with FluidLBM(case, storage=storage, layout=layout) as sim:
        sim.initialize(rho, case.velocity)
        sim.step(3, residual=True)
        with pytest.raises(capi.LbmNonFinite, match="non-finite") as e:
            sim.residual()
        n = int(re.search(r"(\d+) fluid nodes", str(e.value)).group(1))
        assert n >= 2                       # the seeded nodes, and what they reached
        sim.initialize()                    # the context is intact
        sim.step(3, residual=True)
        r = sim.residual()
        assert np.all(np.isfinite(r))


def test_bounded_host_wait_gives_up_and_the_run_continues():
    """The host's wait on the handle's stream is bounded.  With about 0.1 s of
    queued FP64 steps, a 0.1 ms limit expires and lbm_synchronize returns
    LBM_ERR_TIMEOUT; the queued work is not disturbed: a second wait with a
    long limit succeeds and the fields equal those of a run that was never
    interrupted.  (The work is finite, so nothing can hang.)"""
    case = Case(workloads.cylinder(nx=2048, ny=1024, radius=32.0, center=(512, 515)))
    with FluidLBM(case, storage="fp64") as a, FluidLBM(case, storage="fp64") as b:
        for s in (a, b):
            s.initialize()
            s.step(2)
            s.synchronize()
        a.step(200)
        with pytest.raises(capi.LbmError, match="did not finish") as e:
            a.synchronize(timeout_s=1e-4)
        assert e.value.status == capi.LBM_ERR_TIMEOUT
        a.synchronize(600.0)
        a.step(1, moments=True)
        b.step(201, moments=True)
        ra, ua = a.moments()
        rb, ub = b.moments()
        assert np.array_equal(ra, rb) and np.array_equal(ua, ub)
        assert np.array_equal(a.populations(), b.populations())


def test_device_bounded_wait_gives_up_and_the_handle_stays_usable():
    """A kernel waits on an mbarrier that nothing arrives at, with the bounded
    wait of the pipelined step kernel limited to 20 ms: it gives up, sets the
    handle's error word and returns; the call reports LBM_ERR_TIMEOUT, and the
    handle then steps and reports a finite residual (no fault, no hang)."""
    import ctypes
    case = Case(workloads.cavity(32))
    with FluidLBM(case, storage="fp32_shifted") as sim:
        sim.initialize()
        waited = ctypes.c_double()
        rc = sim.lib.lbm_selftest_bounded_wait(sim.h, 0.02, ctypes.byref(waited))
        assert rc == capi.LBM_ERR_TIMEOUT
        assert "mbarrier" in sim.lib.lbm_last_error().decode()
        assert 0.02 <= waited.value < 1.0
        sim.step(5, residual=True)
        assert np.all(np.isfinite(sim.residual()))
