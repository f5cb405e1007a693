"""CPU restatement of the residual's warp reduction (warp_sum8 in
pylabolt_gb300/csrc/lbm_kernels.cuh): lane l ends with the warp sum of value
(l >> 2) & 7, and lanes 0, 4, ..., 28 between them hold all eight sums."""
import numpy as np


def warp_sum8(v):
    """v: [32 lanes][8] -> [32] per-lane results, the kernel's exchanges."""
    lane = np.arange(32)
    b4, b3, b2 = (lane & 16) != 0, (lane & 8) != 0, (lane & 4) != 0
    a4 = np.empty((32, 4))
    for i in range(4):
        send = np.where(b4, v[:, i], v[:, i + 4])
        keep = np.where(b4, v[:, i + 4], v[:, i])
        a4[:, i] = keep + send[lane ^ 16]
    a2 = np.empty((32, 2))
    for i in range(2):
        send = np.where(b3, a4[:, i], a4[:, i + 2])
        keep = np.where(b3, a4[:, i + 2], a4[:, i])
        a2[:, i] = keep + send[lane ^ 8]
    send = np.where(b2, a2[:, 0], a2[:, 1])
    c = np.where(b2, a2[:, 1], a2[:, 0]) + send[lane ^ 4]
    c = c + c[lane ^ 2]
    c = c + c[lane ^ 1]
    return c


def test_warp_sum8_lane_mapping():
    rng = np.random.default_rng(3)
    v = rng.integers(-1000, 1000, size=(32, 8)).astype(float)   # exact sums
    c = warp_sum8(v)
    want = v.sum(axis=0)
    for lane in range(32):
        assert c[lane] == want[(lane >> 2) & 7]
    assert sorted(((l >> 2) & 7) for l in range(0, 32, 4)) == list(range(8))
