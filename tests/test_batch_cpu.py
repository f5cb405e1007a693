"""Batch packing on the CPU (pylabolt_gb300.batch.shelf_pack): cavities do
not overlap, stay inside the atlas width, start on 32-node boundaries (so
every 32-node row segment belongs to one cavity and can carry its relaxation
rate), and the draw of sizes / Reynolds numbers / lid speeds is seeded."""
import numpy as np
import pytest

from pylabolt_gb300.batch import draw_cavities, shelf_pack


def _check(sides, width):
    off, height = shelf_pack(sides, width)
    owner = -np.ones((width, height), dtype=np.int64)
    for i, (s, (ox, oy)) in enumerate(zip(sides, off)):
        assert ox % 32 == 0
        assert 0 <= ox and ox + s <= width and 0 <= oy and oy + s <= height
        block = owner[ox:ox + s, oy:oy + s]
        assert np.all(block == -1), "overlap"
        block[...] = i
    # one cavity per 32-node row segment
    for y in range(0, height, 7):
        seg = owner[:, y].reshape(-1, 32)
        for row in seg:
            ids = set(row[row >= 0].tolist())
            assert len(ids) <= 1
    return off, height


def test_benchmark_batch_packs():
    sides, res, lids = draw_cavities(256, seed=0)
    assert sides.min() >= 64 and sides.max() <= 512
    assert np.all((res >= 50) & (res <= 1000)) and np.all((lids >= 0.05) & (lids <= 0.1))
    off, height = _check(sides, 8192)
    fill = float((sides.astype(np.int64) ** 2).sum()) / (8192 * height)
    assert fill > 0.6, fill          # shelves, tallest first, keep most of the atlas fluid


def test_draw_is_seeded():
    a = draw_cavities(16, seed=3)
    b = draw_cavities(16, seed=3)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("seed", range(5))
def test_random_sets_pack(seed):
    rng = np.random.default_rng(seed)
    sides = rng.integers(5, 300, size=40)
    _check(sides, 1024)
