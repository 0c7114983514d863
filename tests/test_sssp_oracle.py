"""CPU Dijkstra of the oracle, pinned against scipy's published Dijkstra."""
import numpy as np
import pytest

from oracle import pyoracle


def random_csr(n, m, seed, wmax=1000):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, m)
    dst = rng.integers(0, n, m)
    w = rng.integers(1, wmax + 1, m).astype(np.uint32)
    order = np.lexsort((dst, src))
    src, dst, w = src[order], dst[order], w[order]
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, src + 1, 1)
    return np.cumsum(rowptr), dst.astype(np.int32), w


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_dijkstra_matches_scipy(seed):
    sp = pytest.importorskip("scipy.sparse")
    csg = pytest.importorskip("scipy.sparse.csgraph")
    n, m = 3000, 12000
    rowptr, col, w = random_csr(n, m, seed)
    # scipy keeps the minimum of parallel edges only through an explicit reduction
    mat = sp.csr_matrix((w.astype(np.float64), col, rowptr), shape=(n, n))
    mat.sum_duplicates()
    dup = sp.coo_matrix((w.astype(np.float64), (np.repeat(np.arange(n), np.diff(rowptr)), col)), shape=(n, n))
    best = {}
    for a, b, c in zip(dup.row, dup.col, dup.data):
        best[(a, b)] = min(best.get((a, b), np.inf), c)
    rows, cols = zip(*best.keys())
    mat = sp.csr_matrix((list(best.values()), (rows, cols)), shape=(n, n))
    sources = [0, 17, 2999]
    want = csg.dijkstra(mat, directed=True, indices=sources)
    got = pyoracle.dijkstra(rowptr, col, w, sources, threads=2)
    exp = np.where(np.isinf(want), 0xFFFFFFFF, want).astype(np.uint64)
    assert np.array_equal(got.astype(np.uint64), exp)


def test_dijkstra_unreachable_and_threads():
    rowptr = np.array([0, 1, 1, 1], np.int64)  # 0 -> 1 ; 2 isolated
    col = np.array([1], np.int32)
    w = np.array([7], np.uint32)
    d = pyoracle.dijkstra(rowptr, col, w, [0, 2], threads=4)
    assert d.tolist() == [[0, 7, 0xFFFFFFFF], [0xFFFFFFFF, 0xFFFFFFFF, 0]]
