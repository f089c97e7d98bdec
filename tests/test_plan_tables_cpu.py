"""The vectorised enumerations of the plan tables (GEMM tiles, FP32 staging cells,
combination row chunks) against the nested loops they replace, on random task tables with
empty, ragged and multi-tile tasks."""
import numpy as np
import pytest

from tnkit_gb300 import plan as P
from tnkit_gb300._lib import CVT_ITEM, GEMM_SEG, GEMM_TASK, GEMM_TILE, COMB_ITEM


def _loop_tiles(tasks, segs, tile):
    out, cost = [], []
    for t, task in enumerate(tasks):
        m, n = int(task["m"]), int(task["n"])
        ktot = int(segs[int(task["seg_begin"]):int(task["seg_end"])]["k"].sum()) or 1
        for m0 in range(0, m, tile):
            for n0 in range(0, n, tile):
                out.append((t, m0, n0, 0))
                cost.append(ktot)
    order = np.argsort(-np.asarray(cost, np.int64), kind="stable") if out else []
    return np.array([out[i] for i in order], dtype=GEMM_TILE) if out else np.zeros(0, GEMM_TILE)


def _loop_cvt(tasks):
    items = [(t, r0, c0, 0) for t, (_, _, rows, cols, *_r) in enumerate(tasks)
             for r0 in range(0, rows, 32) for c0 in range(0, cols, 32)]
    return np.array(items, dtype=CVT_ITEM) if items else np.zeros(0, CVT_ITEM)


def _loop_comb_items(tasks):
    items = []
    for t, (_, rows, cols, *_r) in enumerate(tasks):
        step = max(1, P.COMB_CHUNK // max(1, cols))
        for r0 in range(0, rows, step):
            items.append((t, r0, min(rows, r0 + step), 0))
    return np.array(items, dtype=COMB_ITEM) if items else np.zeros(0, COMB_ITEM)


@pytest.mark.parametrize("seed", range(6))
def test_vectorised_tables_match_loops(seed):
    rng = np.random.default_rng(seed)
    nt = int(rng.integers(0, 40))
    dims = lambda: int(rng.choice([0, 1, 7, 63, 64, 65, 128, 129, 300]))
    segs, tasks = [], []
    for t in range(nt):
        b = len(segs)
        for _ in range(int(rng.integers(0, 4))):
            segs.append((0, 0, 1, 1, 1, 1, int(rng.integers(0, 200)), 0, 0, 0, 0, 1.0))
        tasks.append((0, 1, dims(), dims(), b, len(segs), 0))
    ta = np.array(tasks, dtype=GEMM_TASK) if tasks else np.zeros(0, GEMM_TASK)
    sa = np.array(segs, dtype=GEMM_SEG) if segs else np.zeros(0, GEMM_SEG)
    for tile in (64, 128):
        assert np.array_equal(P._tiles(ta, sa, tile), _loop_tiles(ta, sa, tile))
    cvt = [(0, 0, dims(), dims(), 0, 0, 0, 0) for _ in range(nt)]
    assert np.array_equal(P._cvt_items(cvt), _loop_cvt(cvt))
    c = P.CombTable()
    for _ in range(nt):
        c.add(0, dims() * int(rng.integers(1, 300)), dims(), 1, 1, [])
    assert np.array_equal(c.arrays()[2], _loop_comb_items(c.tasks))
