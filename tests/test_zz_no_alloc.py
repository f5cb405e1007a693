"""lbm_conservation_noalloc: the entry point for callers that cannot allocate
device memory (for example code embedded in an application that hands out
all device memory from its own pool).

The test is the caller: it owns the input and output device buffers (through
torch) and calls the entry point through the C-ABI.  The result must match
lbm_conservation, the allocating entry point, on the same populations, within
the FP64 round-off of a differently ordered sum -- on two calls in a row, and
for FP64, FP32-shifted and FP16-shifted views of the populations (the
reduced storages within the rounding of their stored values).

The file name makes pytest collect it last."""
import ctypes

import numpy as np
import pytest

from _golden import load_golden
from pylabolt_gb300 import capi
from pylabolt_gb300.config import Case
from pylabolt_gb300.lbm import FluidLBM

pytestmark = pytest.mark.gpu

RTOL_FP64 = 1e-12      # same populations, different summation order
RTOL_FP32 = 1e-6       # populations rounded to FP32 shifted storage
FP16_SCALE = 4096.0    # FP16 view stores g * scale


def _soa_view(pop_padded, nx, ny):
    """Padded AoS [(nx+2)*(ny+2)][9] -> dense SoA [9][ny][nx] (x fastest)."""
    p = pop_padded.reshape(nx + 2, ny + 2, 9)[1:-1, 1:-1, :]
    return np.ascontiguousarray(p.transpose(2, 1, 0))


def _noalloc(lib, soa, exclude, precision, torch, fp16_scale=0.0):
    dev = torch.device("cuda:0")
    pop_d = torch.from_numpy(soa).to(dev)
    excl_d = torch.from_numpy(exclude).to(dev)
    out_d = torch.full((3,), float("nan"), dtype=torch.float64, device=dev)
    nq, ny, nx = soa.shape
    view = capi.LbmPopView(precision=precision, nx=nx, ny=ny, reserved=0, pitch=nx,
                           plane=ny * nx, pop=pop_d.data_ptr(), exclude=excl_d.data_ptr(),
                           fp16_scale=fp16_scale)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.lbm_conservation_noalloc(ctypes.byref(view), ctypes.c_void_p(out_d.data_ptr()),
                                      ctypes.c_void_p(stream))
    assert rc == capi.LBM_OK, lib.lbm_last_error().decode()
    torch.cuda.synchronize(dev)
    return out_d.cpu().numpy()


def test_noalloc_conservation_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    case = Case(load_golden("channel_cylinder_abb")[0])
    nx, ny = case.nx, case.ny
    exclude = np.ascontiguousarray(case.solid.T.astype(np.uint8))   # [ny][nx]
    with FluidLBM(case, storage="fp64") as sim:
        sim.initialize()
        for steps in (7, 13):                       # two calls in a row
            sim.step(steps)
            ref = sim.conservation()                # lbm_conservation (allocating)
            soa = _soa_view(sim.populations(), nx, ny)
            got = _noalloc(lib, soa, exclude, capi.LBM_FP64, torch)
            np.testing.assert_allclose(got, ref, rtol=RTOL_FP64, atol=1e-13 * abs(ref[0]))
            g = soa - np.array(capi_weights())[:, None, None]
            g32 = g.astype(np.float32)
            got32 = _noalloc(lib, g32, exclude, capi.LBM_FP32_SHIFTED, torch)
            np.testing.assert_allclose(got32, ref, rtol=RTOL_FP32, atol=1e-6 * abs(ref[0]))
            # FP16: each stored g * scale is rounded to half (relative 2^-11 at
            # most, absolute 2^-25 for subnormals), so every sum is within
            # 2^-11 sum |g| + count 2^-25 / scale of the FP64 one
            g16 = (g * FP16_SCALE).astype(np.float16)
            got16 = _noalloc(lib, g16, exclude, capi.LBM_FP16_SHIFTED, torch, FP16_SCALE)
            gk = g[:, exclude == 0]
            bound = (2.0 ** -11 * np.abs(gk).sum() + gk.size * 2.0 ** -25 / FP16_SCALE
                     + 1e-12 * abs(ref[0]))
            np.testing.assert_allclose(got16, ref, rtol=0, atol=bound)


def test_noalloc_rejects_too_many_rows():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    big = capi.NOALLOC_MAX_ROWS + 1
    pop_d = torch.zeros(9 * big * 4, dtype=torch.float64, device="cuda:0")
    out_d = torch.zeros(3, dtype=torch.float64, device="cuda:0")
    view = capi.LbmPopView(precision=capi.LBM_FP64, nx=4, ny=big, reserved=0, pitch=4,
                           plane=4 * big, pop=pop_d.data_ptr(), exclude=None, fp16_scale=0.0)
    rc = lib.lbm_conservation_noalloc(ctypes.byref(view), ctypes.c_void_p(out_d.data_ptr()), None)
    assert rc == capi.LBM_ERR_ARG
    assert "exceeds" in lib.lbm_last_error().decode()


def capi_weights():
    from pylabolt_gb300.lattice import W
    return W
