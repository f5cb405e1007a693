"""D2Q9 lattice constants (pylabolt/base/lattice.py:41-60)."""
import numpy as np

CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.int64)
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], dtype=np.int64)
W = np.array([4 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 9, 1 / 36, 1 / 36, 1 / 36, 1 / 36],
             dtype=np.float64)
INV = np.array([0, 3, 4, 1, 2, 7, 8, 5, 6], dtype=np.int64)

# computed the way the reference computes them in FP64 (lattice.py:41-44):
# inv_cs_2 = 2.999999999999999, inv_cs_4 = 8.999999999999995
CS = np.float64(1 / np.sqrt(3))
CS_2 = CS * CS
INV_CS_2 = 1.0 / CS_2
INV_CS_4 = INV_CS_2 * INV_CS_2
EPS64 = np.finfo(np.float64).eps

# boundary location -> (inward normal, out_list, inv_list), boundary.py:63-78
LOCATIONS = {
    "bottom": ((0, 1), (4, 7, 8), (2, 5, 6)),
    "top": ((0, -1), (2, 5, 6), (4, 7, 8)),
    "left": ((1, 0), (3, 6, 7), (1, 8, 5)),
    "right": ((-1, 0), (1, 8, 5), (3, 6, 7)),
}
