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
    s = new_server(graphs, maps, arena_bytes=2 << 20, max_slots=64, batch_size=bs, variant=variant,
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
