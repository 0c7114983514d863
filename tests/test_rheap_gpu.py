"""GPU tests of the retrieving heap (include/gpuheap_retrieve.cuh,
gh_rheap_*), the in-place partial retrieval of the reference's SSSP
application (applications/sssp_longfei_new/heap.cuh:79-382,
heap_with_aux.cuh:48-119, sssp.cu:19-132).

Bar: bit-exact.  One block replays the reference's own insert / retrieve
sequences (tests/golden/retrieve_ref_cases.npz): every returned run and
count, and the heap each sequence leaves (valid nodes, partial buffer,
counters) equal the reference's.  Concurrent inserts and retrieves in one
launch keep every key exactly once, each retrieved run ascending, and a
valid heap; retrieves that meet an insert still on its way to the last
node take its batch through the root (counted).  SSSP through the
auxiliary buffer equals Dijkstra."""
import numpy as np
import pytest

import golden_cases
from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
from gpuheap_gb300 import rheap as grh  # noqa: E402
from gpuheap_gb300 import sssp as gsssp  # noqa: E402

NP = {"u32": np.uint32, "u64": np.uint64}
TV = {"u32": (np.int32, torch.int32), "u64": (np.int64, torch.int64)}


@pytest.fixture(scope="module", autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield


def dev(a, key):
    return torch.from_numpy(np.ascontiguousarray(a).view(TV[key][0])).cuda()


def host(t, key):
    return t.cpu().numpy().view(NP[key])


@pytest.mark.parametrize("i", range(len(golden_cases.retrieve_meta())))
def test_golden_replay_bit_exact(i):
    c = golden_cases.retrieve_case(i)
    key, B, bn = c["key"], c["batch_size"], c["batch_num"]
    keys_d = dev(c["keys"], key)
    out = torch.zeros(B, dtype=TV[key][1], device="cuda")
    runs, taken, pos = [], [], 0
    with grh.RetrievingHeap(bn, B, key=key) as h:
        for op in c["ops"]:
            if op > 0:
                h.insert(keys_d[pos:pos + op])
                pos += int(op)
            else:
                n = h.retrieve(out, -int(op))
                taken.append(n)
                runs.append(host(out, key)[:n].copy())
        items, pb, st = h.state()
    assert st["error"] == 0
    assert np.array_equal(np.asarray(taken, np.int32), c["taken"])
    assert np.array_equal(np.concatenate(runs), c["runs"])
    bc, ps = st["batch_count"], st["pb_size"]
    assert [bc, ps] == list(c["final_counters"])
    assert np.array_equal(items[:bc * B], c["final_nodes"])
    assert np.array_equal(pb[:ps], c["final_pb"])


def check_heap(items, pb, st, B):
    """Every valid node sorted, a parent's keys not above its children's,
    the partial buffer sorted and not below the root."""
    bc, ps = st["batch_count"], st["pb_size"]
    nodes = items[:bc * B].reshape(bc, B) if bc else np.zeros((0, B), items.dtype)
    for i in range(bc):
        assert np.all(nodes[i][:-1] <= nodes[i][1:]), f"node {i} unsorted"
        for c in (2 * i + 1, 2 * i + 2):
            if c < bc:
                assert nodes[i][-1] <= nodes[c][0], f"node {i} above child {c}"
    assert np.all(pb[:ps][:-1] <= pb[:ps][1:])
    if bc and ps:
        assert nodes[0][-1] <= pb[0]


def drain(h, B, key):
    out = torch.zeros(B, dtype=TV[key][1], device="cuda")
    got = []
    while True:
        n = h.retrieve(out, B)
        if n == 0:
            return got
        run = host(out, key)[:n].copy()
        assert np.all(run[:-1] <= run[1:])
        got.append(run)


@pytest.mark.parametrize("key,B,chunk,size,ins,ret", [
    ("u64", 64, 64, 64, 8, 8), ("u64", 64, 37, 23, 6, 10), ("u32", 128, 128, 100, 16, 4),
    ("u32", 32, 32, 32, 24, 24), ("u64", 256, 256, 256, 12, 12)])
def test_concurrent_inserts_and_retrieves(key, B, chunk, size, ins, ret):
    n = 1 << 16
    keys = pyoracle.gen(key, B + chunk, "uniform", n)
    out = torch.zeros(n, dtype=TV[key][1], device="cuda")
    runs = torch.zeros(2 * (n + 1), dtype=torch.int32, device="cuda")
    with grh.RetrievingHeap(4 * n // B + 16, B, key=key) as h:
        n_out, n_runs = h.concurrent(dev(keys, key), chunk, ins, ret, size, out, runs)
        items, pb, st = h.state()
        assert st["error"] == 0
        check_heap(items, pb, st, B)
        o, r = host(out, key)[:n_out], runs.cpu().numpy()[:2 * n_runs].reshape(-1, 2)
        for at, ln in r:
            assert 0 < ln <= size and np.all(o[at:at + ln - 1] <= o[at + 1:at + ln])
        rest = drain(h, B, key)
    got = np.concatenate([o] + rest)
    assert np.array_equal(np.sort(got), np.sort(keys))


def test_retrieves_take_inserts_in_flight():
    """Full-batch inserts racing retrieves of whole batches on a shallow
    heap: some retrieves find the last node still an insert's target and
    take its batch through the root; the keys all come out exactly once."""
    key, B, n = "u64", 64, 1 << 15
    steals = 0
    for seed in range(6):
        keys = pyoracle.gen(key, 300 + seed, "uniform", n)
        out = torch.zeros(n, dtype=torch.int64, device="cuda")
        runs = torch.zeros(2 * (n + 1), dtype=torch.int32, device="cuda")
        with grh.RetrievingHeap(4 * n // B + 16, B, key=key) as h:
            n_out, n_runs = h.concurrent(dev(keys, key), B, 16, 16, B, out, runs)
            items, pb, st = h.state()
            assert st["error"] == 0
            check_heap(items, pb, st, B)
            got = np.concatenate([host(out, key)[:n_out]] + drain(h, B, key))
            assert np.array_equal(np.sort(got), np.sort(keys))
            steals += st["steals"]
    assert steals > 0


def test_full_heap_refuses_and_reports():
    B = 32
    with grh.RetrievingHeap(4, B, key="u32") as h:
        keys = dev(np.arange(B, dtype=np.uint32), "u32")
        for _ in range(4):
            h.insert(keys)
        items, pb, st = h.state()
        assert st["full"] >= 1 and st["error"] == 2 and st["batch_count"] == 3


@pytest.mark.parametrize("scale,B,chunk,blocks", [(12, 64, 8, 1), (12, 256, 32, 16), (14, 256, 16, 32), (14, 1024, 64, 8)])
def test_sssp_retrieve_matches_dijkstra(scale, B, chunk, blocks):
    g = gsssp.rmat_graph(scale, 16, seed=40 + scale)
    rowptr, col, w = g.host()
    for src in (0, 17, g.n // 2 + 3):
        dist, stats = gsssp.sssp_retrieve(g, src, batch_size=B, chunk=chunk, blocks=blocks)
        want = pyoracle.dijkstra(rowptr, col, w, [src])[0]
        assert np.array_equal(dist.cpu().numpy().view(np.uint32), want)
        assert stats["keys_taken"] > 0
