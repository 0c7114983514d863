"""Served SSSP and grid A* queries on the GPU (gh_serve_*): every result in
a Poisson stream equals the CPU oracle (Dijkstra distances, A* path cost),
and equals the same query run alone; admission waits for free memory."""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
from gpuheap_gb300 import batch as gb  # noqa: E402
from gpuheap_gb300 import serve as gs  # noqa: E402
from gpuheap_gb300 import sssp as gsssp  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield


@pytest.fixture(scope="module")
def datasets():
    graphs = [gsssp.rmat_graph(s, 16, seed=500 + s) for s in (10, 12, 14)]
    maps = [gb.gen_grid(side, 600 + side, height=side // 2 + 7) for side in (64, 200, 511)]
    return graphs, maps


def make_queries(graphs, maps, count, seed):
    rng = np.random.default_rng(seed)
    qs = []
    for _ in range(count):
        if rng.random() < 0.5:
            gi = int(rng.integers(len(graphs)))
            qs.append((gs.SSSP, gi, int(rng.integers(graphs[gi].n)), 0))
        else:
            mi = int(rng.integers(len(maps)))
            cells = maps[mi].size
            qs.append((gs.ASTAR, len(graphs) + mi, int(rng.integers(cells)), int(rng.integers(cells))))
    return qs


def oracle(graphs, maps, qs):
    out = []
    hosts = [g.host() for g in graphs]
    for k, d, a, b in qs:
        if k == gs.SSSP:
            dist = pyoracle.dijkstra(*hosts[d], [a])[0]
            fin = dist != 0xFFFFFFFF
            out.append((int(fin.sum()), int(dist[fin].astype(np.uint64).sum())))
        else:
            out.append((int(pyoracle.astar_grid_sg(maps[d - len(graphs)], a, b)), 0))
    return out


def new_server(graphs, maps, **kw):
    s = gs.Server(**kw)
    for g in graphs:
        s.add_graph(g)
    for m in maps:
        s.add_map(torch.from_numpy(m).cuda())
    return s


def test_served_stream_matches_oracle_and_alone(datasets):
    graphs, maps = datasets
    qs = make_queries(graphs, maps, 60, 1)
    want = oracle(graphs, maps, qs)
    s = new_server(graphs, maps, arena_bytes=1 << 30, max_slots=16, batch_size=256, batches_per_step=2)
    try:
        lat, res, makespan, steps = gs.run_stream(s, qs, gs.poisson_arrivals(len(qs), 400.0, 3))
        assert all(r[0] == gs.FINISHED for r in res)
        assert [(r[1], r[2]) for r in res] == want
        assert np.all(lat > 0) and steps >= 2
        assert s.info()["used_bytes"] == 0 and s.info()["slots_used"] == 0
    finally:
        s.close()
    alone = new_server(graphs, maps, arena_bytes=1 << 30, max_slots=1, batch_size=256, batches_per_step=1 << 20)
    try:
        _, res1 = gs.run_plain(alone, qs[:20])
        assert [(r[1], r[2]) for r in res1] == want[:20]
    finally:
        alone.close()


@pytest.mark.parametrize("variant,bs", [("topdown", 128), ("bottomup", 512)])
def test_admission_waits_for_memory(datasets, variant, bs):
    """An arena that holds about two of the largest queries: the rest wait and
    are admitted as memory frees up, all results exact."""
    graphs, maps = datasets
    qs = make_queries(graphs, maps, 24, 7)
    want = oracle(graphs, maps, qs)
    s = new_server(graphs, maps, arena_bytes=5 << 20, max_slots=64, batch_size=bs, variant=variant,
                   batches_per_step=4)
    try:
        ids = [s.submit(*q) for q in qs]
        peak_queued = 0
        for _ in range(100000):
            fin, active, queued = s.step()
            peak_queued = max(peak_queued, queued)
            if active == 0 and queued == 0:
                break
        res = [s.result(q) for q in ids]
        assert [(r[1], r[2]) for r in res] == want
        assert peak_queued > 0  # memory, not slots, held some back
        assert s.info()["used_bytes"] == 0
    finally:
        s.close()


def test_edge_queries(datasets):
    graphs, maps = datasets
    g = gsssp.rmat_graph(10, 8, seed=3)
    rowptr = g.host()[0]
    iso = np.nonzero(np.diff(rowptr) == 0)[0]
    blocked = gb.gen_grid(40, 9)
    blocked[0, 0] = 0
    s = gs.Server(arena_bytes=256 << 20, max_slots=8, batch_size=64)
    try:
        gi = s.add_graph(g)
        mi = s.add_map(torch.from_numpy(maps[0]).cuda())
        bi = s.add_map(torch.from_numpy(blocked).cuda())
        qs = [(gs.ASTAR, mi, 5, 5), (gs.ASTAR, bi, 0, blocked.size - 1)]
        if iso.size:
            qs.append((gs.SSSP, gi, int(iso[0]), 0))
        ids = [s.submit(*q) for q in qs]
        while True:
            _, active, queued = s.step()
            if active == 0 and queued == 0:
                break
        res = [s.result(q) for q in ids]
        assert res[0][:3] == (gs.FINISHED, 0, 0)
        assert res[1][:3] == (gs.FINISHED, 0xFFFFFFFF, 0)
        if iso.size:
            assert res[2][:3] == (gs.FINISHED, 1, 0)
        with pytest.raises(Exception):
            s.submit(gs.SSSP, mi, 0, 0)  # kind does not match the dataset
        tiny = gs.Server(arena_bytes=16 << 10, max_slots=2, batch_size=64)
        try:
            tiny.add_graph(g)
            with pytest.raises(Exception):
                tiny.submit(gs.SSSP, 0, 0)  # can never fit the arena
        finally:
            tiny.close()
    finally:
        s.close()


# ---------------------------------------------------------------- device loop
def poll_until_done(s, ids, max_seconds=120.0):
    """Polls the device loop until every id has completed; returns the peak
    of `queued` seen."""
    import time
    left = set(ids)
    peak = 0
    t0 = time.perf_counter()
    while left:
        fin, _, queued = s.poll()
        peak = max(peak, queued)
        left -= set(fin)
        assert time.perf_counter() - t0 < max_seconds, f"{len(left)} queries did not complete"
    return peak


def test_device_loop_stream_matches_oracle(datasets):
    """A Poisson stream through the device-resident loop: every result equals
    the oracle, and the arena and slots are free at the end."""
    graphs, maps = datasets
    qs = make_queries(graphs, maps, 60, 11)
    want = oracle(graphs, maps, qs)
    s = new_server(graphs, maps, arena_bytes=1 << 30, max_slots=16, batch_size=256, batches_per_step=2)
    try:
        s.start(idle_ms=200)
        lat, res, makespan, polls = gs.run_stream(s, qs, gs.poisson_arrivals(len(qs), 400.0, 5), resident=True)
        assert all(r[0] == gs.FINISHED for r in res)
        assert [(r[1], r[2]) for r in res] == want
        assert sorted(r[3] for r in res) == list(range(1, len(qs) + 1))  # completion order
        info = s.info()
        assert info["used_bytes"] == 0 and info["slots_used"] == 0 and info["steps"] >= 1
        with pytest.raises(Exception):
            s.step()  # host steps are off once the device loop runs
    finally:
        s.close()


@pytest.mark.parametrize("variant,bs", [("topdown", 128), ("bottomup", 512)])
def test_device_loop_admission_waits_for_memory(datasets, variant, bs):
    """An arena that holds about two of the largest queries: the device
    admits the rest as memory frees up, in arrival order where they fit."""
    graphs, maps = datasets
    qs = make_queries(graphs, maps, 24, 7)
    want = oracle(graphs, maps, qs)
    s = new_server(graphs, maps, arena_bytes=5 << 20, max_slots=64, batch_size=bs, variant=variant,
                   batches_per_step=4)
    try:
        s.start(idle_ms=200)
        ids = [s.submit(*q) for q in qs]
        peak = poll_until_done(s, ids)
        res = [s.result(q) for q in ids]
        assert [(r[1], r[2]) for r in res] == want
        assert peak > 0  # memory, not slots, held some back
        assert s.info()["used_bytes"] == 0
    finally:
        s.close()


def test_device_loop_idle_exit_relaunch_and_stop(datasets):
    """The loop's launch leaves after its idle limit and poll() launches it
    again for new work; stop() pauses it mid-stream and start() resumes the
    queries it left, all results exact."""
    import time
    graphs, maps = datasets
    qs = make_queries(graphs, maps, 40, 21)
    want = oracle(graphs, maps, qs)
    s = new_server(graphs, maps, arena_bytes=1 << 30, max_slots=8, batch_size=256, batches_per_step=1)
    try:
        s.start(idle_ms=5)
        a = s.submit(*qs[0])
        poll_until_done(s, [a])
        time.sleep(0.2)  # well past the idle limit: the launch has left
        s.poll()
        first = s.info()["steps"]
        b = s.submit(*qs[1])
        poll_until_done(s, [b])
        assert s.info()["steps"] == first + 1
        rest = [s.submit(*q) for q in qs[2:]]
        for _ in range(3):
            s.poll()
        s.stop()
        time.sleep(0.05)
        fin, _, _ = s.poll()  # paused: collects what completed, launches nothing
        steps = s.info()["steps"]
        time.sleep(0.05)
        assert s.poll()[0] == [] and s.info()["steps"] == steps
        pending = [q for q in rest if s.result(q)[0] not in (gs.FINISHED, gs.FAILED)]
        assert pending  # the pause left work in the loop
        s.start()
        poll_until_done(s, pending)
        ids = [a, b] + rest
        res = [s.result(q) for q in ids]
        assert all(r[0] == gs.FINISHED for r in res)
        assert [(r[1], r[2]) for r in res] == want
    finally:
        s.close()


def test_device_loop_edge_queries(datasets):
    """Start == goal, a blocked start cell and an isolated vertex through the
    device loop."""
    graphs, maps = datasets
    g = gsssp.rmat_graph(10, 8, seed=3)
    rowptr = g.host()[0]
    iso = np.nonzero(np.diff(rowptr) == 0)[0]
    blocked = gb.gen_grid(40, 9)
    blocked[0, 0] = 0
    s = gs.Server(arena_bytes=256 << 20, max_slots=8, batch_size=64)
    try:
        gi = s.add_graph(g)
        mi = s.add_map(torch.from_numpy(maps[0]).cuda())
        bi = s.add_map(torch.from_numpy(blocked).cuda())
        s.start(idle_ms=50)
        qs = [(gs.ASTAR, mi, 5, 5), (gs.ASTAR, bi, 0, blocked.size - 1)]
        if iso.size:
            qs.append((gs.SSSP, gi, int(iso[0]), 0))
        ids = [s.submit(*q) for q in qs]
        poll_until_done(s, ids)
        res = [s.result(q) for q in ids]
        assert res[0][:3] == (gs.FINISHED, 0, 0)
        assert res[1][:3] == (gs.FINISHED, 0xFFFFFFFF, 0)
        if iso.size:
            assert res[2][:3] == (gs.FINISHED, 1, 0)
    finally:
        s.close()


def test_device_loop_needs_an_idle_server(datasets):
    graphs, maps = datasets
    s = new_server(graphs, maps, arena_bytes=64 << 20, max_slots=4, batch_size=64)
    try:
        s.submit(gs.ASTAR, len(graphs), 0, 1)
        with pytest.raises(Exception):
            s.start()  # a query waits for a host step
        with pytest.raises(Exception):
            s.poll()  # not started
    finally:
        s.close()


@pytest.mark.parametrize("resident", [False, True])
def test_bitmap_maps_on_the_reference_model(datasets, resident):
    """Maps on the reference's own model (gh_serve_add_bitmap: eight moves
    with its direction costs) next to cost grids and graphs, through host
    steps and through the device loop: every A* result equals the optimum
    of the 8-neighbour oracle from its start to its goal."""
    graphs, maps = datasets
    rng = np.random.default_rng(44)
    bitmaps = []
    for k, (w, h) in enumerate([(64, 40), (300, 171), (17, 1)]):
        o = (rng.random((h, w)) >= [0.2, 0.3, 0.0][k]).astype(np.uint8)
        bitmaps.append(o)
    s = new_server(graphs, maps, arena_bytes=1 << 30, max_slots=16, batch_size=256, batches_per_step=2)
    try:
        ids8 = [s.add_bitmap(torch.from_numpy(o).cuda()) for o in bitmaps]
        if resident:
            s.start(idle_ms=100)
        qs, want = [], []
        for j in range(24):
            bi = j % len(bitmaps)
            o = bitmaps[bi]
            a, b = int(rng.integers(o.size)), int(rng.integers(o.size))
            qs.append((gs.ASTAR, ids8[bi], a, b))
            want.append(pyoracle.astar_grid8_sg(o, a, b))
        mixed = make_queries(graphs, maps, 10, 45)
        want += [w for w, _ in oracle(graphs, maps, mixed)]
        qs += mixed
        lat, res, _, _ = gs.run_stream(s, qs, gs.poisson_arrivals(len(qs), 500.0, 9), resident=resident)
        assert all(r[0] == gs.FINISHED for r in res)
        assert [r[1] for r in res] == want
    finally:
        s.close()
