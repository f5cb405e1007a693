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
