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
