"""Every load the step kernels issue stays inside the population allocation.

Restates, on the CPU, the index arithmetic of the layout (planes of (ny+2)
rows of `pitch` elements, one guard row before and after the nine planes) and
of the TMA kernel's bulk-copy windows [x0 - H, x0 + W + H) of rows y - c_y,
for grids that exercise padding, narrow rows and FP32 / FP16 storage."""
import pytest

CY = [0, 0, 1, 0, -1, 1, 1, -1, -1]
TMA_ROW_BYTES, HALO_BYTES = 4096, 16


def layout(nx, ny, eb, fp64=False):
    align = (512 if fp64 else TMA_ROW_BYTES) // eb
    pitch = (nx + align - 1) // align * align
    return pitch, (ny + 2) * pitch


@pytest.mark.parametrize("nx,ny", [(8192, 2048), (4096, 1024), (24, 16), (1000, 7), (12, 10), (3, 3)])
@pytest.mark.parametrize("eb", [4, 2])
def test_tma_windows_inside_allocation(nx, ny, eb):
    pitch, plane = layout(nx, ny, eb)
    W, H = TMA_ROW_BYTES // eb, HALO_BYTES // eb
    lo, hi = -pitch, 9 * plane + pitch          # allocation, relative to plane 0
    assert pitch % W == 0
    for nopull in (False, True):
        for y in (0, ny - 1):
            for x0 in range(0, pitch, W):
                for k in range(9):
                    dy = 0 if nopull else CY[k]
                    src = k * plane + (y + 1) * pitch + x0 - dy * pitch - H
                    assert lo <= src and src + W + 2 * H <= hi
                    assert (src * eb) % 16 == 0 and ((W + 2 * H) * eb) % 16 == 0


@pytest.mark.parametrize("nx,ny", [(8192, 2048), (24, 16), (5, 4)])
@pytest.mark.parametrize("eb,fp64", [(8, True), (4, False), (2, False)])
def test_shifted_pulls_inside_allocation(nx, ny, eb, fp64):
    """Vector / scalar pulls of rows y-1..y+1 and columns x-1..x+V (lane 0 /
    lane 31 extra elements) of every node of every row."""
    pitch, plane = layout(nx, ny, eb, fp64)
    lo, hi = -pitch, 9 * plane + pitch
    for k in range(9):
        for y in (0, ny - 1):
            row = k * plane + (y + 1 - CY[k]) * pitch
            assert lo <= row - 1 and row + pitch + 1 <= hi


CX = [0, 1, 0, -1, 0, 1, -1, -1, 1]


@pytest.mark.parametrize("nx,ny", [(8192, 2048), (4096, 1024), (100, 40), (64, 8), (33, 5)])
@pytest.mark.parametrize("eb", [4, 2])
def test_node_pair_words_inside_allocation(nx, ny, eb):
    """The node-pair kernel's fast path serves a pair only when its whole
    32-node segment is bulk, which keeps it off the domain edges (edge nodes
    always have link records): x0 >= 32 and x0 + 1 <= nx - 2, 1 <= y <= ny - 2.
    Its words (two elements each, element 2w and 2w + 1 of the plane array)
    are then the pulls at r - 1, r, r + 1 with r = k plane/2 - c_ky pitch/2 + w0
    and the stores at k plane/2 + w0, w0 = ((y + 1) pitch + x0) / 2."""
    pitch, plane = layout(nx, ny, eb)
    assert pitch % 2 == 0 and plane % 2 == 0
    lo, hi = -pitch, 9 * plane + pitch
    segs = [s for s in range((nx + 31) // 32) if 32 * s >= 1 and 32 * s + 31 <= nx - 2]
    if not segs or ny < 3:
        return
    for y in (1, ny - 2):
        for s in (segs[0], segs[-1]):
            for x0 in (32 * s, 32 * s + 30):
                w0 = ((y + 1) * pitch + x0) // 2
                for k in range(9):
                    r = k * (plane // 2) - CY[k] * (pitch // 2) + w0
                    words = {0: [r], 1: [r - 1, r], -1: [r, r + 1]}[CX[k]]
                    words.append(k * (plane // 2) + w0)
                    for w in words:
                        assert lo <= 2 * w and 2 * w + 1 < hi
                    # the two values used are the nodes' own sources
                    src = k * plane + (y + 1 - CY[k]) * pitch + x0 - CX[k]
                    used = {0: (2 * r, 2 * r + 1), 1: (2 * r - 1, 2 * r),
                            -1: (2 * r + 1, 2 * r + 2)}[CX[k]]
                    assert used == (src, src + 1)
