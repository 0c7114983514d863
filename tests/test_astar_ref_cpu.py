"""The oracle's A* machinery pinned to the reference's own sequential A*
(artifacts/astar/seq_astar.hpp:85-183, SeqAstarSearch): on 40 seeded
bitmaps (sides 1-200, obstacle shares 0-45 %; tests/golden/
astar_ref_cases.npz, made by tests/golden/make_golden.py from the reference
compiled on the host) the restatement of its 8-connected move model
(oracle/search_oracle.cpp gho_astar_ref8) returns the reference's result in
every case.  The project's 4-connected cost-grid A* (gho_astar_grid_sg) is
the same closed-set search with another move model and the goal taken when
popped; where the reference's host build exists it is also run directly."""
import ctypes
import json
import os

import numpy as np
import pytest

from oracle import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = np.load(os.path.join(HERE, "golden", "astar_ref_cases.npz"))
META = json.loads(bytes(DATA["meta"]).decode())


@pytest.mark.parametrize("i", range(len(META)))
def test_restatement_matches_the_reference(i):
    m = META[i]
    words, want = DATA[f"c{i}_words"], int(DATA[f"c{i}_result"][0])
    assert pyoracle.astar_ref8(words, m["width"], m["height"]) == want


def test_cases_cover_reached_and_unreached_corners():
    res = [int(DATA[f"c{i}_result"][0]) for i in range(len(META))]
    assert any(r == 0xFFFFFFFF for r in res) and sum(r != 0xFFFFFFFF for r in res) >= 20


@pytest.mark.parametrize("i", range(0, len(META), 5))
def test_reference_host_run_reproduces_the_vectors(i):
    lib_path = os.path.join(os.path.dirname(pyoracle.HERE), "oracle", "_ref", "libbgpq_ref.so")
    if not os.path.exists(lib_path):
        pytest.skip("reference heaps not built here (set GH_REFERENCE_TREE for build())")
    ref = ctypes.CDLL(lib_path)
    if not hasattr(ref, "ra_seq_astar"):
        pytest.skip("reference build without the sequential A*")
    fn = ref.ra_seq_astar
    fn.restype = ctypes.c_uint32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]
    m = META[i]
    words = np.ascontiguousarray(DATA[f"c{i}_words"], np.uint32)
    assert fn(ctypes.c_void_p(words.ctypes.data), m["height"], m["width"]) == int(DATA[f"c{i}_result"][0])


def test_optimal_eight_neighbour_oracle_equals_dijkstra():
    """gho_astar_grid8 (the reference's map model searched to the optimum,
    the result of its GPU A*) against scipy's Dijkstra on the same graph."""
    sp = pytest.importorskip("scipy.sparse")
    cg = pytest.importorskip("scipy.sparse.csgraph")
    dx, dy, cost = [-1, 0, 1, -1, 1, -1, 0, 1], [-1, -1, -1, 0, 0, 1, 1, 1], [3, 2, 2, 2, 1, 3, 1, 2]
    rng = np.random.default_rng(5)
    for _ in range(120):
        w, h = int(rng.integers(1, 25)), int(rng.integers(1, 25))
        o = (rng.random((h, w)) >= rng.choice([0.0, 0.2, 0.4])).astype(np.uint8)
        o[0, 0] = o[-1, -1] = 1
        rows, cols, vals = [], [], []
        for y in range(h):
            for x in range(w):
                if not o[y, x]:
                    continue
                for k in range(8):
                    nx, ny = x + dx[k], y + dy[k]
                    if 0 <= nx < w and 0 <= ny < h and o[ny, nx]:
                        rows.append(y * w + x)
                        cols.append(ny * w + nx)
                        vals.append(cost[k])
        g = sp.csr_matrix((vals, (rows, cols)), shape=(w * h, w * h))
        d = cg.dijkstra(g, indices=0)[-1]
        want = 0xFFFFFFFF if np.isinf(d) else int(d)
        assert pyoracle.astar_grid8(o) == want
