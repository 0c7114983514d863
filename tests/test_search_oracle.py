"""CPU checks of the search oracles (grid A*, knapsack branch-and-bound) and
of the host-side grid generator."""
import numpy as np
import pytest

from oracle import pyoracle


def grid_dijkstra(cost, start=0, goal=None):
    """Independent check: scipy Dijkstra on the grid's move graph."""
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    h, w = cost.shape
    idx = np.arange(h * w).reshape(h, w)
    rows, cols, vals = [], [], []
    for dy, dx in ((0, 1), (0, -1), (1, 0), (-1, 0)):
        ys, xs = np.mgrid[0:h, 0:w]
        ny, nx = ys + dy, xs + dx
        ok = (ny >= 0) & (ny < h) & (nx >= 0) & (nx < w)
        src = idx[ok]
        dst = idx[ny[ok], nx[ok]]
        c = cost.ravel()[dst]
        keep = (c > 0) & (cost.ravel()[src] > 0)
        rows.append(src[keep]); cols.append(dst[keep]); vals.append(c[keep].astype(np.float64))
    m = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(h * w, h * w))
    goal = h * w - 1 if goal is None else goal
    if cost.ravel()[start] == 0:
        return 0xFFFFFFFF
    d = csgraph.dijkstra(m, indices=start)[goal]
    return 0xFFFFFFFF if not np.isfinite(d) else int(d)


@pytest.mark.parametrize("shape,obst,seed", [((1, 1), 0.0, 0), ((1, 9), 0.0, 1), ((7, 1), 0.0, 2), ((5, 5), 0.2, 3),
                                             ((30, 40), 0.2, 4), ((64, 64), 0.35, 5), ((20, 20), 0.6, 6)])
def test_astar_oracle_matches_dijkstra(shape, obst, seed):
    rng = np.random.default_rng(seed)
    cost = rng.integers(1, 10, shape).astype(np.uint8)
    cost[rng.random(shape) < obst] = 0
    cost[0, 0] = max(cost[0, 0], 1)
    cost[-1, -1] = max(cost[-1, -1], 1)
    assert pyoracle.astar_grid(cost) == grid_dijkstra(cost)


@pytest.mark.parametrize("seed", range(4))
def test_astar_oracle_any_start_and_goal(seed):
    rng = np.random.default_rng(40 + seed)
    h, w = int(rng.integers(3, 40)), int(rng.integers(3, 40))
    cost = rng.integers(1, 10, (h, w)).astype(np.uint8)
    cost[rng.random((h, w)) < 0.25] = 0
    for _ in range(5):
        s, g = (int(x) for x in rng.integers(0, h * w, 2))
        assert pyoracle.astar_grid_sg(cost, s, g) == (0 if s == g and cost.ravel()[s] else grid_dijkstra(cost, s, g))


def test_astar_oracle_unreachable_and_blocked():
    cost = np.ones((5, 5), np.uint8)
    cost[:, 2] = 0  # a wall
    assert pyoracle.astar_grid(cost) == 0xFFFFFFFF
    cost = np.ones((3, 3), np.uint8)
    cost[0, 0] = 0
    assert pyoracle.astar_grid(cost) == 0xFFFFFFFF
    assert pyoracle.astar_grid(np.full((1, 1), 7, np.uint8)) == 0


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (10, 2), (40, 3), (100, 4), (300, 5)])
def test_knapsack_bb_matches_dp(n, seed):
    rng = np.random.default_rng(seed)
    w = rng.integers(1, 1001, n).astype(np.int32)
    p = (w + rng.integers(0, 101, n)).astype(np.int32)
    for cap in (0, int(w.min()) - 1, int(w.sum()) // 2, int(w.sum()), int(w.sum()) + 5):
        cap = max(cap, 0)
        assert pyoracle.knap_bb(w, p, cap) == pyoracle.knap_dp(w, p, cap)


def test_knapsack_many_and_astar_many():
    rng = np.random.default_rng(9)
    inst = []
    for n in (5, 50, 120):
        w = rng.integers(1, 1001, n).astype(np.int32)
        p = (w + rng.integers(0, 101, n)).astype(np.int32)
        inst.append((w, p, int(w.sum()) // 2))
    got = pyoracle.knap_bb_many(inst, threads=2)
    assert list(got) == [pyoracle.knap_dp(*x) for x in inst]
    grids = []
    for s in (3, 17, 33):
        g = rng.integers(1, 10, (s, s + 2)).astype(np.uint8)
        grids.append(g)
    assert list(pyoracle.astar_grid_many(grids, threads=2)) == [pyoracle.astar_grid(g) for g in grids]


def test_grid_generator(ghlib):
    from gpuheap_gb300 import batch
    a = batch.gen_grid(300, 11)
    b = batch.gen_grid(300, 11)
    c = batch.gen_grid(300, 12)
    assert a.shape == (300, 300) and a.dtype == np.uint8
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a[0, 0] > 0 and a[-1, -1] > 0
    assert a.max() <= 9
    frac = np.mean(a == 0)
    assert 0.18 < frac < 0.22
    free = a[a > 0]
    assert free.min() == 1 and abs(free.mean() - 5.0) < 0.1
    r = batch.gen_grid(50, 3, height=20, obstacle_per_mille=0)
    assert r.shape == (20, 50) and r.min() >= 1


def test_knapsack_generator():
    from gpuheap_gb300 import batch
    w, p, cap = batch.gen_knapsack(500, 4)
    assert w.min() >= 1 and w.max() <= 1000
    assert np.all(p - w >= 0) and np.all(p - w <= 100)
    assert cap == int(w.sum()) // 2
