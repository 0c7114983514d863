"""GPU tests of the bulk delete's owner mode (k_delete_owner): one block keeps
node 0 and the top levels of the heap in shared memory and merges every level
of a delete's path at once, worker blocks continue each sift below it.

Bar: bit-exact.  Every deleted stream equals the sorted keys.  A bulk delete
stopped by its output limit leaves a heap that checkInsertHeap accepts, with
the right counters, from which the rest comes out in order.  Random heaps put
back from host memory (gh_heap_restore) give every order relation between
the carried batch (the last node) and the children on the path, so the
general sift step (heap/tditdd/heap.cuh:418-532: children merge, then the
case analysis against the carried batch) runs at the resident levels, not
only the fast path that a heap-sort of uniform keys takes.
"""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402

TORCH_VIEW = {"u32": (np.int32, torch.int32), "i32": (np.int32, torch.int32), "u64": (np.int64, torch.int64)}
NP_KEY = {"u32": np.uint32, "i32": np.int32, "u64": np.uint64}
INIT = {"u32": np.uint32(0xFFFFFFFF), "i32": np.int32(0x7FFFFFFF), "u64": np.uint64(0xFFFFFFFFFFFFFFFF)}


@pytest.fixture(scope="module", autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield


def to_dev(a, key):
    return torch.from_numpy(np.ascontiguousarray(a).view(TORCH_VIEW[key][0])).cuda()


def to_host(t, key):
    return t.cpu().numpy().view(NP_KEY[key])


def batch_num_for(n, B):
    bn = 1
    while bn * B < 2 * n:
        bn <<= 1
    return bn


def parent_of(i, variant):
    if variant == "topdown":
        return i >> 1
    r = pyoracle.reversed_idx
    return r(r(i) >> 1)


def random_heap(variant, key, B, bc, batch_num, ps, seed):
    """A valid heap of bc full nodes (and ps partial-buffer keys) whose nodes
    draw their keys above their parent's last key with spreads from one
    batch to millions, so that subtrees interleave in every way."""
    rng = np.random.default_rng(seed)
    dt = NP_KEY[key]
    items = np.full((batch_num + 1) * B, INIT[key], dtype=dt)
    last = {}
    for i in range(1, bc + 1):  # a parent's index is below its children's in both layouts
        base = 0 if i == 1 else int(last[parent_of(i, variant)])
        span = int(rng.choice([B, 16 * B, 4096 * B, 1 << 22]))
        off = int(rng.choice([0, 0, int(rng.integers(0, 1 << 20))]))
        vals = np.sort(base + off + rng.integers(0, span, B)).astype(dt)
        items[i * B:(i + 1) * B] = vals
        last[i] = vals[-1]
    if ps:
        items[:ps] = np.sort(int(last[1]) + rng.integers(0, 1 << 22, ps)).astype(dt)
    ok, msg = pyoracle.check_heap(variant, items, None, B, bc, ps)
    assert ok, msg
    return items


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("pb", [True, False])
@pytest.mark.parametrize("key,B", [("u32", 2048), ("u32", 1024), ("u64", 2048), ("i32", 512), ("u64", 1024)])
def test_partial_bulk_deletes(variant, pb, key, B):
    """Bulk deletes cut by their output limit: after each one the heap passes
    checkInsertHeap and holds the rest; all pieces together are sorted."""
    n = (1 << 20) + (B // 3 if pb else 0)
    keys = pyoracle.gen(key, 5 + B, "uniform", n)
    h = gh.Heap(batch_num_for(n, B), B, key=key, variant=variant, partial_buffer=pb)
    h.insert(to_dev(keys, key), chunk=B)
    h.sync()
    out = torch.zeros(n, dtype=TORCH_VIEW[key][1], device="cuda")
    pieces, left = [], n
    for k in (37, 101, 5, 211):
        got = h.delete(out, max_keys=k * B + B // 2)
        assert got == k * B
        pieces.append(to_host(out, key)[:got].copy())
        left -= got
        assert h.item_count() == left
        ok, msg = h.check_insert_heap()
        assert ok, msg
    assert h.delete(out) == left
    pieces.append(to_host(out, key)[:left].copy())
    st = h.owner_stats()
    h.close()
    assert np.array_equal(np.concatenate(pieces), np.sort(keys))
    assert st["deletes"] > 0 and st["lends"] > 0  # the last bulk delete ran in owner mode


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("key,B", [("u32", 512), ("u32", 2048), ("u64", 1024), ("i32", 1024)])
@pytest.mark.parametrize("ps", [0, 77])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_restored_random_heaps(variant, key, B, ps, seed):
    """Random valid heaps: the bulk delete takes every key out in order, also
    when stopped halfway and resumed."""
    bc, batch_num = 150 + 37 * seed, 512
    items = random_heap(variant, key, B, bc, batch_num, ps, seed * 1000 + B + ps)
    want = np.sort(np.concatenate([items[:ps], items[B:(bc + 1) * B]]))
    total = bc * B + ps
    out = torch.zeros(total, dtype=TORCH_VIEW[key][1], device="cuda")
    with gh.Heap(batch_num, B, key=key, variant=variant, partial_buffer=True) as h:
        h.restore(items, [bc, ps, 0])
        assert h.delete(out) == total
        assert np.array_equal(to_host(out, key), want)
        h.restore(items, [bc, ps, 0])
        first = h.delete(out, max_keys=40 * B)
        assert first == 40 * B
        head = to_host(out, key)[:first].copy()
        ok, msg = h.check_insert_heap()
        assert ok, msg
        assert h.delete(out) == total - first
        assert np.array_equal(np.concatenate([head, to_host(out, key)[:total - first]]), want)


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("key,B", [("u32", 512), ("u32", 2048), ("u64", 1024)])
def test_general_step_runs(variant, key, B):
    """Among a few random heaps at least one makes the owner take the general
    sift step at a resident level (its counter), with the output in order."""
    bc, batch_num = 200, 512
    total = bc * B
    out = torch.zeros(total, dtype=TORCH_VIEW[key][1], device="cuda")
    with gh.Heap(batch_num, B, key=key, variant=variant, partial_buffer=True) as h:
        for seed in range(12):
            items = random_heap(variant, key, B, bc, batch_num, 0, 7000 + seed)
            h.restore(items, [bc, 0, 0])
            assert h.delete(out) == total
            assert np.array_equal(to_host(out, key), np.sort(items[B:(bc + 1) * B]))
            if h.owner_stats()["general_steps"] > 0:
                return
    pytest.fail("no general sift step in 12 random heaps")


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("grid", [2, 3, 8])
def test_few_workers(variant, grid):
    """The owner with one, two or seven worker blocks: lends wait for a free
    worker, lent nodes come back, the output is the same."""
    B, n = 1024, 1 << 19
    keys = pyoracle.gen("u32", grid, "uniform", n)
    with gh.Heap(batch_num_for(n, B), B, key="u32", variant=variant) as h:
        h.set_grid(grid)
        out = torch.zeros(n, dtype=torch.int32, device="cuda")
        h.sort(to_dev(keys, "u32"), out)
        assert np.array_equal(to_host(out, "u32"), np.sort(keys))


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
def test_reserved_insert_then_single_ops(variant):
    """Bulk inserts of full batches take reserved targets; the heap they leave
    is valid, and single insertion()/deleteRoot calls work on it after."""
    B = 512
    n = 300 * B
    keys = pyoracle.gen("u32", 77, "uniform", n + B)
    with gh.Heap(batch_num_for(n + B, B), B, key="u32", variant=variant) as h:
        h.insert(to_dev(keys[:n], "u32"), chunk=B)
        h.sync()
        ok, msg = h.check_insert_heap()
        assert ok, msg
        assert h.node_count() == 300
        h.insertion(to_dev(keys[n:], "u32"), B)
        out = torch.zeros(n + B, dtype=torch.int32, device="cuda")
        assert h.delete_root(out) == B
        first = to_host(out, "u32")[:B].copy()
        assert h.delete(out) == n
        got = np.concatenate([first, to_host(out, "u32")[:n]])
        assert np.array_equal(got, np.sort(keys))
