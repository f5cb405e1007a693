"""Every load the step kernels issue stays inside the population allocation.

Restates, on the CPU, the index arithmetic of the layout (planes of (ny+2)
rows of `pitch` elements, one guard row before and after the nine planes) and
of the node-pair tile kernel's bulk-copy windows [x0 - H, x0 + TW + H) of rows
y - c_y and shared-memory words, for grids that exercise padding, narrow rows
and FP32 / FP16 storage."""
import pytest

CX = [0, 1, 0, -1, 0, 1, -1, -1, 1]
CY = [0, 0, 1, 0, -1, 1, 1, -1, -1]
TMA_ROW_BYTES, HALO_BYTES = 4096, 16


def layout(nx, ny, eb, fp64=False):
    align = (512 if fp64 else TMA_ROW_BYTES) // eb
    pitch = (nx + align - 1) // align * align
    return pitch, (ny + 2) * pitch


TILE_BYTES, SMEM_PER_SM = 2048, 228 * 1024


@pytest.mark.parametrize("nx,ny", [(8192, 2048), (4096, 1024), (2144, 70), (24, 16), (1000, 7),
                                   (12, 10), (3, 3)])
@pytest.mark.parametrize("eb", [4, 2])
def test_tile_windows_inside_allocation(nx, ny, eb):
    """The node-pair tile kernel (kind 2) copies, for tile (y, x0), the rows
    y - c_ky of every plane over [x0 - H, x0 + TW + H): TW = 2048 bytes of
    nodes, x0 a multiple of TW below nx, H one 16-byte granule."""
    pitch, plane = layout(nx, ny, eb)
    TW, H = TILE_BYTES // eb, HALO_BYTES // eb
    lo, hi = -pitch, 9 * plane + pitch          # allocation, relative to plane 0
    assert pitch % TW == 0
    tpr = (nx + TW - 1) // TW
    for y in (0, ny - 1):
        for x0 in range(0, tpr * TW, TW):
            for k in range(9):
                src = k * plane + (y + 1) * pitch + x0 - CY[k] * pitch - H
                assert lo <= src and src + TW + 2 * H <= hi
                assert (src * eb) % 16 == 0 and ((TW + 2 * H) * eb) % 16 == 0


INV = [0, 3, 4, 1, 2, 7, 8, 5, 6]


@pytest.mark.parametrize("nx,ny", [(8192, 2048), (2144, 70), (1000, 33), (100, 7), (24, 16),
                                   (3, 3)])
@pytest.mark.parametrize("eb", [4, 2])
def test_aa_tile_windows_inside_allocation(nx, ny, eb):
    """The tile kernel in the AA layout: rows padded to 128 bytes with at
    least one padding column (not whole tiles), copies of [x0 - H,
    x0 + w + H) with w = min(TW, nx rounded up to the granule - x0): plane k
    of row y in the even phase, plane kbar of row y - c_ky in the odd one."""
    align = 128 // eb
    pitch = (nx + 1 + align - 1) // align * align
    plane = (ny + 2) * pitch
    TW, H = TILE_BYTES // eb, HALO_BYTES // eb
    nxr = (nx + H - 1) // H * H
    lo, hi = -pitch, 9 * plane + pitch
    tpr = (nx + TW - 1) // TW
    for y in (0, ny - 1):
        for x0 in range(0, tpr * TW, TW):
            w = min(TW, nxr - x0)
            assert w >= min(TW, nx - x0) and (w + 2 * H) * eb % 16 == 0
            for k in range(9):
                for src in ((k * plane + (y + 1) * pitch + x0 - H),
                            (INV[k] * plane + (y + 1 - CY[k]) * pitch + x0 - H)):
                    assert lo <= src and src + w + 2 * H <= hi
                    assert (src * eb) % 16 == 0


@pytest.mark.parametrize("eb", [4, 2])
@pytest.mark.parametrize("ppt", [1, 2, 4])
def test_tile_shared_words_and_blocks(eb, ppt):
    """Shared-memory words a pair reads stay inside its stage row, and they
    hold the pulled nodes x - c_kx; the blocks the grid formula asks for fit
    one SM's shared memory, and the contiguous tile ranges cover every tile
    once."""
    TW, H = TILE_BYTES // eb, HALO_BYTES // eb
    RWW = (TW + 2 * H) // 2
    block = TW // (2 * ppt)
    for j in range(TW // 2):
        wi = H // 2 + j
        for k in range(9):
            words = [wi] if CX[k] == 0 else ([wi - 1, wi] if CX[k] == 1 else [wi, wi + 1])
            assert all(0 <= w < RWW for w in words)
            # elements (low, high) the pair takes: mid() = high half of the
            # first word, low half of the second
            got = [2 * wi, 2 * wi + 1] if CX[k] == 0 else [2 * words[0] + 1, 2 * words[1]]
            assert got == [2 * j + d - CX[k] + H for d in (0, 1)]
    for stages, res in ((1, False), (2, True), (3, False), (3, True), (4, False)):
        stage = 9 * (TW + 2 * H) * eb
        # stages, the full/empty barriers, the residual rows (16 warps x 8
        # doubles) of a residual launch, the runtime's 1 KB per block
        smem = stages * stage + 2 * 8 * 8 + (16 * 8 * 8 if res else 0) + 1024
        per_sm = max(min(SMEM_PER_SM // smem, 1024 // block), 1)
        assert stages * stage <= 227 * 1024
        assert per_sm * smem <= SMEM_PER_SM or per_sm == 1
        for ntiles in (1, 7, 16384):
            grid = min(152 * per_sm, ntiles)
            cover = []
            for b in range(grid):
                cover += range(ntiles * b // grid, ntiles * (b + 1) // grid)
            assert cover == list(range(ntiles))


@pytest.mark.parametrize("nx,ny", [(8192, 2048), (24, 16), (5, 4)])
@pytest.mark.parametrize("eb,fp64", [(8, True), (4, False), (2, False)])
def test_shifted_pulls_inside_allocation(nx, ny, eb, fp64):
    """Scalar pulls of rows y-1..y+1 and columns x-1..x+1 of every node of
    every row."""
    pitch, plane = layout(nx, ny, eb, fp64)
    lo, hi = -pitch, 9 * plane + pitch
    for k in range(9):
        for y in (0, ny - 1):
            row = k * plane + (y + 1 - CY[k]) * pitch
            assert lo <= row - 1 and row + pitch + 1 <= hi


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
