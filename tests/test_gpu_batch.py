"""Batched cavities (pylabolt_gb300.batch): the atlas case against each cavity
run on its own, and the omega map's validation."""
import numpy as np
import pytest

from pylabolt_gb300 import capi, workloads
from pylabolt_gb300.batch import CavityBatch, draw_cavities
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu


def test_batch_equals_single_cavities():
    # small cavities at moderate Re (Re/N <= 6, tau >= 0.53): stable with BGK
    sides, res, lids = draw_cavities(n=10, seed=3, side=(48, 96), re=(50.0, 300.0))
    steps = 300
    with CavityBatch(sides, res, lids, width=256) as b:
        b.initialize()
        b.step(steps, moments=True)
        ub = b.velocities()
    for i in range(len(sides)):
        case = Case(workloads.cavity(int(sides[i]), re=float(res[i]), lid=float(lids[i])))
        with FluidLBM(case, storage="fp32_shifted") as s:
            s.initialize()
            s.step(steps, moments=True)
            _, u = s.moments()
        assert np.abs(ub[i] - u).max() <= 1e-6 * np.abs(u).max()
        with FluidLBM(case, storage="fp64") as s:
            s.initialize()
            s.step(steps, moments=True)
            _, u64 = s.moments()
        # FP32 storage vs FP64: worst node at the singular lid corners
        assert np.abs(ub[i] - u64).max() <= 3e-5 * np.abs(u64).max()


def _fp64_velocities(sides, res, lids, steps):
    """Each cavity on its own FP64 handle; the handles' steps are queued on
    their own streams before any result is read, so they run side by side."""
    sims = []
    try:
        for i in range(len(sides)):
            case = Case(workloads.cavity(int(sides[i]), re=float(res[i]), lid=float(lids[i])))
            s = FluidLBM(case, storage="fp64")
            sims.append(s)
            s.initialize()
            s.step(steps, moments=True)
        return [s.moments()[1] for s in sims]
    finally:
        for s in sims:
            s.close()


def test_c4_distribution_32_cavities_vs_fp64():
    """The first 32 cavities of the benchmark's draw (sides U{64..512}, Re
    U[50, 1000], lid U[0.05, 0.1], seed 0) batched in FP32 shifted storage
    against each cavity run alone in FP64."""
    sides, res, lids = draw_cavities()
    sides, res, lids = sides[:32], res[:32], lids[:32]
    steps = 1000
    with CavityBatch(sides, res, lids) as b:
        b.initialize()
        b.step(steps, moments=True)
        ub = b.velocities()
    u64 = _fp64_velocities(sides, res, lids, steps)
    errs = [np.abs(ub[i] - u64[i]).max() / np.abs(u64[i]).max() for i in range(len(sides))]
    assert max(errs) <= 1e-5, max(errs)


def test_omega_map_rejects_mixed_segment():
    case = Case(workloads.cavity(64))
    with FluidLBM(case, storage="fp32_shifted") as s:
        om = np.full(64 * 64, case.omega)
        om[5] = 1.0          # node (0, 5) differs from the rest of its segment
        with pytest.raises(capi.LbmError, match="segment"):
            s.lib.lbm_set_omega_map and capi.check(s.lib.lbm_set_omega_map(s.h, capi.ptr(om)))
