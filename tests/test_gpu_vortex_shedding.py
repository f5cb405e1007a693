"""Vortex shedding behind a cylinder: the lift and drag from the
momentum-exchange forces (pylabolt/parallel/cpu/force_torque_kernels.py:11-92)
of a developed Re = 100 wake.

Channel 800 x 200, velocity inlet u = 0.1 (moving-wall bounce-back),
anti-bounce-back outlet, bounce-back walls, cylinder of diameter D = 20 at
(160, 101) (blockage 0.1), MRT.  After 20,000 steps of development the lift
is sampled every 10 steps for 20,000 more.  Its dominant frequency f gives the
Strouhal number St = f D / u (0.19, resolution 0.01 from the 20,000-step
window), the mean drag the coefficient Cd = 2 Fx / (u^2 D) (1.74) and the lift
range the amplitude of Cl (0.46).  The bounds are the physical range of a
confined cylinder wake at Re 100 (an unconfined one sheds at St 0.16-0.17,
and blockage raises St and Cd); FP32 storage must give FP64's numbers to
1e-5, FP16 within 3 %."""
import numpy as np
import pytest

from pylabolt_gb300 import workloads
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

D, U, EVERY, DEVELOP, SAMPLES = 20, 0.1, 10, 2000, 2000


def _wake(storage):
    case = Case(workloads.cylinder_shedding(diameter=D, u_in=U))
    lift, drag = [], []
    with FluidLBM(case, storage=storage) as sim:
        sim.initialize()
        sim.step(DEVELOP * EVERY)
        for _ in range(SAMPLES):
            sim.step(EVERY)
            f = sim.forces()["obstacles"][0]
            drag.append(f[0])
            lift.append(f[1])
    lift, drag = np.array(lift), np.array(drag)
    spec = np.abs(np.fft.rfft((lift - lift.mean()) * np.hanning(len(lift))))
    freq = np.fft.rfftfreq(len(lift), d=float(EVERY))
    st = freq[1 + np.argmax(spec[1:])] * D / U
    cd = 2.0 * drag.mean() / (U * U * D)
    cl = (lift.max() - lift.min()) / (U * U * D)
    return st, cd, cl


def test_strouhal_and_drag_of_the_wake():
    st, cd, cl = _wake("fp64")
    assert 0.16 <= st <= 0.22, st
    assert 1.4 <= cd <= 2.0, cd
    assert 0.3 <= cl <= 0.6, cl
    st32, cd32, cl32 = _wake("fp32_shifted")
    assert st32 == st
    assert abs(cd32 - cd) <= 1e-5 * cd and abs(cl32 - cl) <= 1e-5 * cl
    st16, cd16, cl16 = _wake("fp16_shifted")
    assert abs(st16 - st) <= 0.0101
    assert abs(cd16 - cd) <= 0.03 * cd and abs(cl16 - cl) <= 0.03 * cl
