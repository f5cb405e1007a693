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


def test_omega_map_rejects_mixed_segment():
    case = Case(workloads.cavity(64))
    with FluidLBM(case, storage="fp32_shifted") as s:
        om = np.full(64 * 64, case.omega)
        om[5] = 1.0          # node (0, 5) differs from the rest of its segment
        with pytest.raises(capi.LbmError, match="segment"):
            s.lib.lbm_set_omega_map and capi.check(s.lib.lbm_set_omega_map(s.h, capi.ptr(om)))
