"""A large grid against a small one: 16384 x 8192 FP32-shifted lid-driven
cavity (population buffers of 4.8 GB, byte offsets beyond 2^32, node indices
up to 1.3e8) and a 256 x 192 cavity with the same viscosity, lid and launch
shape.  Information moves one node per step, so after T steps the windows at
the lid's corners and at its middle, more than T nodes from every other wall,
hold the same values in both grids, bit for bit.  Mass is conserved in the
closed cavity.  About 20 GB of device memory."""
import numpy as np
import pytest

from pylabolt_gb300 import workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

T = 24
W = 40        # window width / height (> T: the window's far edge is untouched too)
MASS_RTOL = 1e-6


def _run(nx, ny):
    # re = nx: nu = 0.1 * nx / nx = 0.1 exactly for power-of-two nx
    case = Case(workloads.cavity(nx, re=float(nx), storage="fp32_shifted", ny=ny))
    with FluidLBM(case) as sim:
        sim.initialize()
        m0 = sim.conservation()[0]
        sim.step(T, moments=True)
        m1 = sim.conservation()[0]
        rho, u = sim.moments()
    return rho, u, m0, m1


def _windows(rho, u):
    nx, ny = rho.shape
    mid = nx // 2
    out = []
    for xs in (slice(0, W), slice(mid - W // 2, mid + W // 2), slice(nx - W, nx)):
        out.append((rho[xs, ny - W:], u[xs, ny - W:]))
    return out


def test_large_grid_windows_match_small_grid(monkeypatch):
    monkeypatch.setenv("LBM_VARIANT", "0,1,128,1")
    big = _run(16384, 8192)
    small = _run(256, 192)
    for (rb, ub), (rs, us) in zip(_windows(*big[:2]), _windows(*small[:2])):
        assert np.array_equal(rb, rs)
        assert np.array_equal(ub, us)
    assert np.abs(ub).max() > 0          # the lid has set the windows moving
    for _, _, m0, m1 in (big, small):
        assert abs(m1 - m0) <= MASS_RTOL * m0
