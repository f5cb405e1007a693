"""The kernel's closed-form MRT collision (moments, equilibrium moments, Guo
source moments, inverse transform), transcribed line by line, against the
oracle's matrix form M^-1 [m - S(m - M f_eq) + (I - S/2) M Fbar] -- on random
node states, in FP64 (round-off agreement) and in the FP32 shifted form."""
import numpy as np
import pytest
import sympy as sp

from oracle.lbm_np import M_MRT, M_INV, equilibrium
from oracle.setup import CX, CY, W, INV_CS_2, INV_CS_4


def kernel_mrt(f, rho, drho, ux, uy, Fx, Fy, rates, forc, shifted, i2, i4, T):
    """Transcription of mrt_collide in pylabolt_gb300/csrc/lbm_kernels.cuh."""
    f = [T(v) for v in f]
    rho, drho, ux, uy, Fx, Fy = (T(v) for v in (rho, drho, ux, uy, Fx, Fy))
    i2, i4 = T(i2), T(i4)
    s_e, s_eps, s_q, s_nu = (T(v) for v in rates)
    a14 = f[1] + f[2] + f[3] + f[4]
    a58 = f[5] + f[6] + f[7] + f[8]
    m = [f[0] + a14 + a58, T(-4) * f[0] - a14 + T(2) * a58, T(4) * f[0] - T(2) * a14 + a58,
         f[1] - f[3] + f[5] - f[6] - f[7] + f[8],
         T(-2) * f[1] + T(2) * f[3] + f[5] - f[6] - f[7] + f[8],
         f[2] - f[4] + f[5] + f[6] - f[7] - f[8],
         T(-2) * f[2] + T(2) * f[4] + f[5] + f[6] - f[7] - f[8],
         f[1] - f[2] + f[3] - f[4], f[5] - f[6] + f[7] - f[8]]
    u2 = ux * ux + uy * uy
    t2, n4 = i2 / T(3), i4 / T(9)
    meq = [(drho if shifted else rho) - rho * ((T(3) * i2 - i4) / T(6)) * u2,
           (T(-2) * drho + rho * i2 * u2) if shifted else rho * (i2 * u2 - T(2)),
           (drho - rho * ((T(3) * i2 + i4) / T(6)) * u2) if shifted
           else rho - rho * ((T(3) * i2 + i4) / T(6)) * u2,
           t2 * rho * ux, -t2 * rho * ux, t2 * rho * uy, -t2 * rho * uy,
           n4 * rho * (ux * ux - uy * uy), n4 * rho * ux * uy]
    mf = [T(0)] * 9
    if forc:
        mf[3], mf[4], mf[5], mf[6] = t2 * Fx, -t2 * Fx, t2 * Fy, -t2 * Fy
    if forc == 2:
        uF = Fx * ux + Fy * uy
        mf[0] = -((T(3) * i2 - i4) / T(3)) * uF
        mf[1] = T(2) * i2 * uF
        mf[2] = -((T(3) * i2 + i4) / T(3)) * uF
        mf[7] = T(2) * n4 * (Fx * ux - Fy * uy)
        mf[8] = n4 * (Fx * uy + Fy * ux)
    S = [T(1), s_e, s_eps, T(1), s_q, T(1), s_q, s_nu, s_nu]
    inv_norm = [T(1) / T(v) for v in (9, 36, 36, 6, 12, 6, 12, 4, 4)]
    a = [(m[i] - S[i] * (m[i] - meq[i]) + (T(1) - T(0.5) * S[i]) * mf[i]) * inv_norm[i]
         for i in range(9)]
    b = a[0] - a[1] - T(2) * a[2]
    c = a[0] + T(2) * a[1] + a[2]
    return np.array([a[0] - T(4) * a[1] + T(4) * a[2],
                     b + a[3] - T(2) * a[4] + a[7], b + a[5] - T(2) * a[6] - a[7],
                     b - a[3] + T(2) * a[4] + a[7], b - a[5] + T(2) * a[6] - a[7],
                     c + a[3] + a[4] + a[5] + a[6] + a[8], c - a[3] - a[4] + a[5] + a[6] - a[8],
                     c - a[3] - a[4] - a[5] - a[6] + a[8], c + a[3] + a[4] - a[5] - a[6] - a[8]],
                    dtype=np.float64)


def matrix_mrt(f, rho, ux, uy, Fx, Fy, rates, forc):
    s_e, s_eps, s_q, s_nu = rates
    S = np.array([1.0, s_e, s_eps, 1.0, s_q, 1.0, s_q, s_nu, s_nu])
    m = M_MRT @ f
    meq = M_MRT @ equilibrium(np.array([rho]), np.array([ux]), np.array([uy]))[0]
    fb = np.zeros(9)
    for k in range(9):
        cu = CX[k] * ux + CY[k] * uy
        if forc == 1:
            fb[k] = W[k] * (CX[k] * Fx + CY[k] * Fy) * INV_CS_2
        elif forc == 2:
            fb[k] = W[k] * (((CX[k] - ux) * INV_CS_2 + cu * CX[k] * INV_CS_4) * Fx +
                            ((CY[k] - uy) * INV_CS_2 + cu * CY[k] * INV_CS_4) * Fy)
    return M_INV @ (m - S * (m - meq) + (1 - 0.5 * S) * (M_MRT @ fb))


@pytest.mark.parametrize("forc", [0, 1, 2])
def test_closed_form_equals_matrix_form(forc):
    rng = np.random.default_rng(7)
    rates = (1.4, 1.4, 1.2, 0.79)
    for _ in range(200):
        ux, uy = rng.uniform(-0.1, 0.1, 2)
        rho = 1 + rng.uniform(-0.01, 0.01)
        f = equilibrium(np.array([rho]), np.array([ux]), np.array([uy]))[0]
        f = f * (1 + rng.uniform(-0.05, 0.05, 9))
        rho = f.sum()
        Fx, Fy = rng.uniform(-1e-4, 1e-4, 2)
        ref = matrix_mrt(f, rho, ux, uy, Fx, Fy, rates, forc)
        got = kernel_mrt(f, rho, rho, ux, uy, Fx, Fy, rates, forc, False,
                         INV_CS_2, INV_CS_4, np.float64)
        assert np.abs(got - ref).max() < 1e-15
        g = f - W
        got32 = kernel_mrt(g, rho, rho - 1, ux, uy, Fx, Fy, rates, forc, True,
                           3.0, 9.0, np.float32) + W
        assert np.abs(got32 - ref).max() < 3e-8


def test_shifted_mass_deviation_is_kept_below_fp32_spacing_of_one():
    """A mass deviation far below FP32's spacing of 1 (1.2e-7) survives the
    shifted collision: the density moment is never formed as (1 + drho) - 1."""
    drho = 3e-9
    g = W * drho
    out = kernel_mrt(g, 1 + drho, drho, 0.0, 0.0, 0.0, 0.0, (1.4, 1.4, 1.2, 0.8), 0, True,
                     3.0, 9.0, np.float32)
    assert abs(out.sum() - drho) < 1e-12


def test_equilibrium_moments_closed_form_symbolic():
    rho, ux, uy, i2, i4 = sp.symbols("rho ux uy i2 i4")
    Wt = [sp.Rational(4, 9)] + [sp.Rational(1, 9)] * 4 + [sp.Rational(1, 36)] * 4
    u2 = ux ** 2 + uy ** 2
    feq = [Wt[k] * rho * (1 + i2 * (int(CX[k]) * ux + int(CY[k]) * uy) +
                          sp.Rational(1, 2) * i4 * (int(CX[k]) * ux + int(CY[k]) * uy) ** 2 -
                          sp.Rational(1, 2) * i2 * u2) for k in range(9)]
    M = sp.Matrix(M_MRT.astype(int).tolist())
    meq = M * sp.Matrix(feq)
    closed = [rho - rho * (3 * i2 - i4) / 6 * u2, rho * (i2 * u2 - 2),
              rho - rho * (3 * i2 + i4) / 6 * u2, i2 / 3 * rho * ux, -i2 / 3 * rho * ux,
              i2 / 3 * rho * uy, -i2 / 3 * rho * uy, i4 / 9 * rho * (ux ** 2 - uy ** 2),
              i4 / 9 * rho * ux * uy]
    for a in range(9):
        assert sp.simplify(meq[a] - closed[a]) == 0
