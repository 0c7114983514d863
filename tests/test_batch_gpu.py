"""Batched searches on the GPU (gh_batch_*): every instance's result equals
the CPU oracle exactly (A* path costs, knapsack optima), in the persistent,
graph-replayed and plain per-instance forms, run after run."""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402
from gpuheap_gb300 import batch as gb  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield


def small_mix(seed=5):
    rng = np.random.default_rng(seed)
    inst = []
    # edge cases: single cell, single row / column, walled-off goal, blocked start
    inst.append(("astar", np.full((1, 1), 3, np.uint8)))
    inst.append(("astar", gb.gen_grid(37, 1, height=1, obstacle_per_mille=0)))
    inst.append(("astar", gb.gen_grid(1, 2, height=45, obstacle_per_mille=0)))
    wall = gb.gen_grid(40, 3, obstacle_per_mille=0)
    wall[:, 20] = 0
    inst.append(("astar", wall))
    blocked = gb.gen_grid(16, 4)
    blocked[0, 0] = 0
    inst.append(("astar", blocked))
    for i in range(20):
        side = int(rng.integers(8, 300))
        inst.append(("astar", gb.gen_grid(side, 100 + i, height=int(rng.integers(8, 300)))))
    # knapsacks: nothing fits, everything fits, one item, random sizes
    w = np.array([50, 60, 70], np.int32)
    inst.append(("knapsack", (w, w + 5, 10)))
    inst.append(("knapsack", (w, w + 5, 1000)))
    inst.append(("knapsack", (np.array([7], np.int32), np.array([9], np.int32), 7)))
    for i in range(20):
        inst.append(("knapsack", gb.gen_knapsack(int(rng.integers(2, 400)), 200 + i)))
    return inst


def oracle_results(inst):
    grids = [d for k, d in inst if k == "astar"]
    knaps = [d for k, d in inst if k == "knapsack"]
    a = iter(pyoracle.astar_grid_many(grids, threads=8))
    k = iter(pyoracle.knap_bb_many(knaps, threads=8))
    return np.array([int(next(a)) if kind == "astar" else int(next(k)) for kind, _ in inst], np.int64)


@pytest.mark.parametrize("bs,variant", [(64, "bottomup"), (256, "bottomup"), (128, "topdown"), (512, "topdown")])
def test_batch_matches_oracle_every_mode(bs, variant):
    inst = small_mix()
    want = oracle_results(inst)
    b = gb.Batch(inst, batch_size=bs, variant=variant, astar_cells_per_block=1 << 12)
    try:
        for mode in ("persistent", "graph", "graph", "plain", "persistent"):
            b.run(mode)
            res, st, stats = b.results()
            assert not st.any()
            assert np.array_equal(res, want), (mode, np.nonzero(res != want))
            assert np.all(stats[:, 0] >= 0)
    finally:
        b.close()


def test_batch_large_grid_many_blocks():
    """A 1024^2 grid shared by 8 blocks, next to small instances."""
    inst = [("astar", gb.gen_grid(1024, 77)), ("astar", gb.gen_grid(300, 78)),
            ("knapsack", gb.gen_knapsack(1000, 79)), ("knapsack", gb.gen_knapsack(1000, 80))]
    want = oracle_results(inst)
    for variant in ("bottomup", "topdown"):
        b = gb.Batch(inst, batch_size=256, variant=variant, astar_cells_per_block=1 << 17, astar_max_blocks=8)
        try:
            assert b.info()["tasks"] == 8 + 1 + 1 + 1
            for mode in ("graph", "plain"):
                b.run(mode)
                res, st, _ = b.results()
                assert np.array_equal(res, want), (variant, mode)
        finally:
            b.close()


def test_knapsack_matches_dp():
    inst = [("knapsack", gb.gen_knapsack(n, 300 + n)) for n in (1, 3, 17, 64, 150)]
    want = [pyoracle.knap_dp(*d) for _, d in inst]
    b = gb.Batch(inst, batch_size=64)
    try:
        b.run("graph")
        res, _, _ = b.results()
        assert list(res) == want
    finally:
        b.close()


def knapsack_set(ns):
    w = np.array([50, 60, 70], np.int32)
    inst = [("knapsack", (w, w + 5, 10)), ("knapsack", (w, w + 5, 1000)),
            ("knapsack", (np.array([7], np.int32), np.array([9], np.int32), 7))]
    return inst + [("knapsack", gb.gen_knapsack(n, 900 + n)) for n in ns]


# instance sizes whose breadth-first frontier stays far below the 2^20-node
# pool (a CPU breadth-first run of the same instances peaks below 40 K nodes)
FIFO_SIZES = (2, 17, 100, 200, 300, 500)


@pytest.mark.parametrize("order,counter", [("fifo", 20), ("switch", 20), ("switch", 2),
                                           ("switch", 1), ("heap", 20)])
def test_knapsack_orders_match_oracle(order, counter):
    """The knapsack models of the reference -- best-first on the heap,
    breadth-first through the FIFO ring, and the heap/FIFO switch -- all
    reach the CPU branch-and-bound optimum, mixed with A* instances.

    How many switches an instance makes depends on the block schedule (the
    order children reach the queue and the pool slots they get), so only
    their presence is checked: with a short counter at least one instance
    leaves the heap, and with a counter of 1 one also comes back from the
    FIFO ring, over the two runs.  In the batch-synchronous model of these
    instances (oracle/knapsack_orders.py, pinned by
    tests/test_knapsack_orders_cpu.py), a counter of 2 switches each of the
    four largest once and a counter of 1 three times."""
    inst = small_mix(11)[:12] + knapsack_set(FIFO_SIZES)
    want = oracle_results(inst)
    kinds = np.array([k == "knapsack" for k, _ in inst])
    b = gb.Batch(inst, batch_size=128, knapsack_order=order, switch_counter=counter)
    try:
        most = 0
        for mode in ("graph", "plain"):
            b.run(mode)
            res, st, stats = b.results()
            assert not st.any(), st
            assert np.array_equal(res, want), (order, mode, np.nonzero(res != want))
            sw = b.knapsack_switches()
            assert not sw[~kinds].any()
            if order in ("fifo", "heap"):
                assert not sw.any()
            most = max(most, int(sw[kinds].max()))
        if order == "switch" and counter <= 2:
            assert most >= 1, "expected a heap-to-FIFO switch with a short counter"
        if order == "switch" and counter == 1:
            assert most >= 2, "expected a FIFO-to-heap switch with a counter of 1"
    finally:
        b.close()


def test_knapsack_fifo_overflow_is_reported():
    """A breadth-first frontier wider than the node pool (800 items: over 3 M
    nodes on the CPU) fails that instance with GH_ERR_CAPACITY; the other
    instances of the batch still finish with their optimum."""
    inst = knapsack_set((100, 800))
    want = oracle_results(inst)
    b = gb.Batch(inst, batch_size=128, knapsack_order="fifo")
    try:
        b.run("graph")
        res, st, _ = b.results(check=False)
        assert st[-1] == gh.GH_ERR_CAPACITY
        assert not st[:-1].any()
        assert np.array_equal(res[:-1], want[:-1])
    finally:
        b.close()


def test_batch_rejects_bad_arguments():
    with pytest.raises(Exception):
        gb.Batch([("astar", gb.gen_grid(8, 1))], batch_size=100)
    with pytest.raises(Exception):
        gb.Batch([("knapsack", (np.ones(2000, np.int32), np.ones(2000, np.int32), 5))])


@pytest.mark.parametrize("bs,variant", [(64, "bottomup"), (256, "topdown"), (512, "bottomup")])
def test_astar_on_the_reference_map_model(bs, variant):
    """A* instances on the reference's own model (eight neighbours with its
    direction costs over an open/blocked bitmap, gh_batch_add_astar_bitmap)
    next to cost-grid A* and knapsack instances: every result equals the
    optimum of the matching oracle, in every mode."""
    rng = np.random.default_rng(33)
    inst = []
    inst.append(("astar8", np.ones((1, 1), np.uint8)))
    inst.append(("astar8", np.ones((1, 40), np.uint8)))
    walled = np.ones((30, 30), np.uint8)
    walled[:, 15] = 0
    inst.append(("astar8", walled))  # the diagonal moves cannot cross a full wall either
    gap = walled.copy()
    gap[29, 15] = 1
    inst.append(("astar8", gap))
    for i in range(16):
        w, h = int(rng.integers(8, 400)), int(rng.integers(8, 400))
        o = (rng.random((h, w)) >= [0.0, 0.2, 0.35, 0.45][i % 4]).astype(np.uint8)
        o[0, 0] = o[-1, -1] = 1
        inst.append(("astar8", o))
    for i in range(6):
        side = int(rng.integers(8, 200))
        inst.append(("astar", gb.gen_grid(side, 300 + i)))
        inst.append(("knapsack", gb.gen_knapsack(int(rng.integers(2, 200)), 400 + i)))
    want = []
    for kind, d in inst:
        if kind == "astar8":
            want.append(pyoracle.astar_grid8(d))
        elif kind == "astar":
            want.append(int(pyoracle.astar_grid_many([d], threads=1)[0]))
        else:
            want.append(int(pyoracle.knap_bb_many([d], threads=1)[0]))
    want = np.array(want, np.int64)
    assert want[2] == 0xFFFFFFFF and want[3] != 0xFFFFFFFF
    b = gb.Batch(inst, batch_size=bs, variant=variant, astar_cells_per_block=1 << 12)
    try:
        for mode in ("persistent", "graph", "plain"):
            b.run(mode)
            res, st, _ = b.results()
            assert not st.any()
            assert np.array_equal(res, want), (mode, np.nonzero(res != want))
    finally:
        b.close()
