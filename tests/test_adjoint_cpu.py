"""The adjoint's mathematics on the CPU: the plain-torch FP64 reference
gradient against central finite differences, and a line-by-line NumPy
transcription of the CUDA adjoint (tests/_adjoint_emulator.py, same transpose
tables and reverse-mode formulas) against that reference, to round-off."""
import numpy as np
import pytest
import torch

from _adjoint_emulator import adjoint
from _golden import load_golden
from _torch_lbm import TorchLBM
from pylabolt_gb300.config import Case

RTOL = 1e-12


def _body_force_case(forcing, seed=3):
    case_d, _ = load_golden("poiseuille_guo2")
    rng = np.random.default_rng(seed)
    case_d["collision_dict"]["fluid"]["forcing_model"] = forcing
    case_d["forcing_dict"] = {"body_force_field": 1e-5 + 1e-6 * rng.standard_normal((10, 8, 2))}
    return Case(case_d)


def test_torch_reference_against_central_differences():
    case = _body_force_case("guo_second_order")
    tl = TorchLBM(case)
    rng = np.random.default_rng(1)
    F = torch.tensor(case.body_force_field.reshape(-1, 2), requires_grad=True)
    target = torch.tensor(rng.standard_normal((80, 2)) * 1e-4)

    def loss(F):
        u = tl.run(20, torch.tensor(case.omega, dtype=torch.float64), force=F)
        return ((u - target) ** 2).mean()

    loss(F).backward()
    d = torch.tensor(rng.standard_normal(F.shape))
    h = 1e-7
    with torch.no_grad():
        fd = (loss(F + h * d) - loss(F - h * d)) / (2 * h)
    assert abs(float((F.grad * d).sum()) - float(fd)) <= 1e-7 * abs(float(fd))


@pytest.mark.parametrize("forcing", ["guo_second_order", "guo_linear"])
def test_adjoint_transcription_body_force_and_tau(forcing):
    case = _body_force_case(forcing)
    tl = TorchLBM(case)
    F = torch.tensor(case.body_force_field.reshape(-1, 2), requires_grad=True)
    tau = torch.tensor(case.tau, dtype=torch.float64, requires_grad=True)
    u = tl.run(25, 1.0 / tau, force=F)
    gu = np.random.default_rng(2).standard_normal(u.shape) * 1e-3
    (u * torch.tensor(gu)).sum().backward()
    gF, gtau, _ = adjoint(case, 25, gu, force=case.body_force_field.reshape(-1, 2))
    np.testing.assert_allclose(gF, F.grad.numpy(), rtol=0, atol=RTOL * np.abs(F.grad.numpy()).max())
    assert abs(gtau - float(tau.grad)) <= RTOL * abs(float(tau.grad))


@pytest.mark.parametrize("name", ["cavity_lid_last", "periodic_moving_disk"])
def test_adjoint_transcription_wall_velocity_tau_gravity(name):
    case = Case(load_golden(name)[0])
    tl = TorchLBM(case)
    uw = torch.tensor([0.1, 0.0], dtype=torch.float64, requires_grad=True)
    tau = torch.tensor(case.tau, dtype=torch.float64, requires_grad=True)
    u = tl.run(12, 1.0 / tau, u_wall=uw)
    gu = np.random.default_rng(4).standard_normal(u.shape) * 1e-3
    gu[case.solid.ravel()] = 0.0          # the velocity of solid nodes is not an output
    (u * torch.tensor(gu)).sum().backward()
    _, gtau, guw = adjoint(case, 12, gu)
    assert abs(gtau - float(tau.grad)) <= RTOL * abs(float(tau.grad))
    if uw.grad is not None and np.abs(uw.grad.numpy()).max() > 0:
        np.testing.assert_allclose(guw, uw.grad.numpy(), rtol=0,
                                   atol=RTOL * np.abs(uw.grad.numpy()).max())
