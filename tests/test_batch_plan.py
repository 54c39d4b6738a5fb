"""Host-side work list of batched rendering (vsrPlanBatch), no GPU needed:
every pixel of every job is covered by exactly one tile, jobs come in order
of cost per pixel (highest first, stable), tile widths must divide 32."""
import numpy as np
import pytest


def covered(items, widths, heights, tile_w):
    tile_h = 32 // tile_w
    seen = [np.zeros((h, w), np.int32) for w, h in zip(widths, heights)]
    for job, tile in items:
        w, h = widths[job], heights[job]
        tiles_x = (w + tile_w - 1) // tile_w
        tx, ty = tile % tiles_x, tile // tiles_x
        ys = slice(ty * tile_h, min((ty + 1) * tile_h, h))
        xs = slice(tx * tile_w, min((tx + 1) * tile_w, w))
        assert ys.start < h and xs.start < w, "tile outside the frame"
        seen[job][ys, xs] += 1
    return seen


@pytest.mark.parametrize("tile_w", [1, 2, 4, 8, 16, 32])
def test_plan_covers_every_pixel_once(pkg, tile_w):
    widths, heights = [17, 64, 5, 1, 100], [9, 32, 3, 1, 7]
    costs = [1.0, 4.0, 1.0, 2.0, 0.5]
    items = pkg.vsr.plan_batch(widths, heights, costs, tile_w)
    for s in covered(items, widths, heights, tile_w):
        assert (s == 1).all()


def test_plan_orders_jobs_by_cost(pkg):
    widths, heights = [16, 16, 16, 16], [8, 8, 8, 8]
    costs = [1.0, 3.0, 1.0, 2.0]
    items = pkg.vsr.plan_batch(widths, heights, costs, 8)
    order = [int(j) for j in dict.fromkeys(items[:, 0])]
    assert order == [1, 3, 0, 2]   # stable for the two jobs of cost 1
    # all tiles of a job are contiguous and in tile order
    for j in range(4):
        rows = np.nonzero(items[:, 0] == j)[0]
        assert (np.diff(rows) == 1).all()
        assert (items[rows, 1] == np.arange(len(rows))).all()


def test_plan_rejects_bad_tile_width_and_empty_jobs(pkg):
    assert len(pkg.vsr.plan_batch([8], [8], [1.0], 3)) == 0
    assert len(pkg.vsr.plan_batch([0, 8], [5, 4], [1.0, 1.0], 8)) == 1
