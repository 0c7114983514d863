"""GPU parity tests of the CUDA heap through the C ABI.

Bar: bit-exact.  With one thread block the heap is deterministic, so its
memory must equal the reference's own run (golden vectors) and the oracle
model; with many concurrent blocks the deleted stream must equal std::sort
and checkInsertHeap must hold after the insert phase (test/test.sh:5-32).
"""
import numpy as np
import pytest

import golden_cases
from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402

# torch views of the key types (bit patterns, no arithmetic on them)
TORCH_VIEW = {"u32": (np.int32, torch.int32), "i32": (np.int32, torch.int32), "u64": (np.int64, torch.int64)}
NP_KEY = {"u32": np.uint32, "i32": np.int32, "u64": np.uint64}


def to_dev(a, key):
    npv, _ = TORCH_VIEW[key]
    return torch.from_numpy(np.ascontiguousarray(a).view(npv)).cuda()


def empty_dev(n, key):
    return torch.zeros(n, dtype=TORCH_VIEW[key][1], device="cuda")


def to_host(t, key):
    return t.cpu().numpy().view(NP_KEY[key])


def batch_num_for(n, B):
    bn = 1
    while bn * B < 2 * n:
        bn <<= 1
    return bn


@pytest.fixture(scope="module", autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield


@pytest.mark.parametrize("which,i", golden_cases.all_ids())
def test_golden_replay_single_block(which, i):
    """One block replays the reference's operation list; heap memory, counters,
    deleteRoot sizes and the HEAP_SORT stream equal the reference's run.  Both
    sets: batch 16-64 and the configurations' batch sizes 256-2048."""
    c = golden_cases.case(i, which)
    key, B = c["key"], c["batch_size"]
    h = gh.Heap(c["batch_num"], B, key=key, variant="topdown" if c["topdown"] else "bottomup",
                partial_buffer=c["partial_buffer"])
    keys = to_dev(c["keys"], key)
    out = empty_dev(c["out"].size, key)
    pos, dsizes = 0, []
    for op in c["ops"]:
        if op > 0:
            h.insertion(keys[pos:pos + op], int(op))
            pos += op
        elif op == 0:
            dsizes.append(h.delete_root(out))
        else:
            items, status, counters = h.snapshot()
            assert np.array_equal(counters[:3], c["snap_counters"]), "counters after the insert phase"
            assert np.array_equal(items, c["snap_items"]), "heap memory after the insert phase"
            assert not status.any()
            ok, msg = h.check_insert_heap()
            assert ok, msg
    items, status, counters = h.snapshot()
    assert counters[3] == 0, f"device error {counters[3:]}"
    assert dsizes == list(c["dsizes"]), "deleteRoot sizes"
    assert np.array_equal(to_host(out, key), c["out"]), "HEAP_SORT output"
    assert np.array_equal(items, c["items"]), "final heap memory"
    assert np.array_equal(counters[:3], c["counters"]), "final counters"
    h.close()


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("pb", [True, False])
@pytest.mark.parametrize("key,B,threads", [("u32", 256, 0), ("u32", 1024, 0), ("u32", 512, 1024),
                                           ("u32", 512, 128), ("u64", 256, 0), ("i32", 2048, 0)])
def test_random_ops_match_model(variant, pb, key, B, threads):
    """Single block, random insert sizes and interleaved deletes, against the
    oracle model: every node bit-exact at the end."""
    rng = np.random.default_rng(B * 7 + threads + (3 if pb else 0) + (1 if variant == "topdown" else 0))
    nb = 40
    n = nb * B
    bn = batch_num_for(n, B)
    keys = pyoracle.gen(key, int(rng.integers(1 << 30)), "uniform", n)
    h = gh.Heap(bn, B, key=key, variant=variant, partial_buffer=pb)
    if threads:
        h.set_block_threads(threads)
    m = pyoracle.Model(key, variant, pb, bn, B)
    dk = to_dev(keys, key)
    out_d = empty_dev(n + 2 * B, key)
    out_m = np.zeros(n + 2 * B, NP_KEY[key])
    pos = 0
    while True:
        if pos < n and rng.random() < 0.6:
            s = B if not pb else int(rng.integers(1, B + 1))
            s = min(s, n - pos)
            if not pb and s < B:
                pos = n
                continue
            h.insertion(dk[pos:pos + s], s)
            assert m.insert(keys[pos:pos + s]) == 0
            pos += s
        else:
            a = h.delete_root(out_d)
            b = m.delete(out_m)
            assert a == b
            if pos >= n and a == 0:
                break
    items, status, counters = h.snapshot()
    mi, mc = m.state()
    assert np.array_equal(items, mi)
    assert np.array_equal(counters[:3], mc)
    assert np.array_equal(to_host(out_d, key), out_m)
    h.close()


def model_retrieve(m, size, B, dtype):
    """The oracle side of retrieve: a delete of the root batch, the first
    `size` keys returned, the rest inserted back."""
    _, counters = m.state()
    before = int(counters[2])
    buf = np.zeros(before + 2 * B, dtype)
    n = m.delete(buf)
    keys = buf[before:before + n].copy()
    take = min(n, size)
    if n > take:
        assert m.insert(keys[take:]) == 0
    return keys[:take]


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("key,B", [("u32", 256), ("u64", 512), ("i32", 1024)])
def test_retrieve_matches_model(variant, key, B):
    """retrieve(ret, size): random inserts and retrieves of random sizes by one
    block against the oracle (delete the root batch, return the first `size`,
    insert the rest back): every retrieved run and the final heap bit-exact."""
    rng = np.random.default_rng(B + len(variant))
    n = 30 * B
    bn = batch_num_for(n, B)
    keys = pyoracle.gen(key, int(rng.integers(1 << 30)), "uniform", n)
    h = gh.Heap(bn, B, key=key, variant=variant, partial_buffer=True)
    m = pyoracle.Model(key, variant, True, bn, B)
    dk = to_dev(keys, key)
    out_d = empty_dev(B, key)
    pos, got_total = 0, 0
    while True:
        if pos < n and rng.random() < 0.55:
            s = min(int(rng.integers(1, B + 1)), n - pos)
            h.insertion(dk[pos:pos + s], s)
            assert m.insert(keys[pos:pos + s]) == 0
            pos += s
        else:
            size = int(rng.integers(1, B + 1)) if rng.random() < 0.8 else B
            got = h.retrieve(out_d, size)
            want = model_retrieve(m, size, B, NP_KEY[key])
            assert got == len(want)
            assert np.array_equal(to_host(out_d, key)[:got], want)
            got_total += got
            if pos >= n and got == 0:
                break
    assert got_total == n
    items, status, counters = h.snapshot()
    mi, mc = m.state()
    assert np.array_equal(items, mi)
    assert np.array_equal(counters[:2], mc[:2])
    h.close()


def test_retrieve_edges():
    B = 64
    h = gh.Heap(16, B, key="u32", variant="bottomup", partial_buffer=True)
    out = empty_dev(B, "u32")
    assert h.retrieve(out, 10) == 0                     # empty heap
    keys = np.arange(100, 100 + 3 * B + 5, dtype=np.uint32)[::-1].copy()
    h.insert(to_dev(keys, "u32"), chunk=7)
    assert h.retrieve(out, 0) == 0
    assert h.retrieve(out, 5) == 5
    assert np.array_equal(to_host(out, "u32")[:5], np.arange(100, 105))
    assert h.retrieve(out, 10 * B) == B                   # at most one batch
    assert np.array_equal(to_host(out, "u32"), np.arange(105, 105 + B))
    assert h.item_count() == 3 * B + 5 - 5 - B
    ok, msg = h.check_insert_heap()
    assert ok, msg
    h.close()
    h = gh.Heap(16, B, key="u32", variant="topdown", partial_buffer=False)
    with pytest.raises(gh.HeapError) as e:
        h.retrieve(out, 5)
    assert e.value.status == gh.GH_ERR_INVALID
    h.close()


def run_heap_sort(key, variant, pb, B, n, dist="uniform", seed=1, chunk=None, grid=0):
    keys = pyoracle.gen(key, seed, dist, n)
    h = gh.Heap(batch_num_for(n, B), B, key=key, variant=variant, partial_buffer=pb)
    if grid:
        h.set_grid(grid)
    dk = to_dev(keys, key)
    out = empty_dev(n, key)
    h.insert(dk, chunk=chunk if chunk is not None else (B // 3 if pb else B))
    h.sync()
    ok, msg = h.check_insert_heap()
    assert ok, msg
    assert h.item_count() == n
    got_n = h.delete(out)
    assert got_n == n
    assert h.is_empty()
    got = to_host(out, key)
    want = pyoracle.sort(keys.copy(), threads=8)
    h.close()
    return got, want


# test/test.sh:5-32: B in {128..1024} x N in {2^20, 2^21, 2^22} x the four variants
@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("pb", [True, False])
@pytest.mark.parametrize("B", [128, 256, 512, 1024])
@pytest.mark.parametrize("logn", [20, 21, 22])
def test_heap_sort_grid(variant, pb, B, logn):
    n = (2**logn + B - 1) // B * B
    got, want = run_heap_sort("u32", variant, pb, B, n, seed=logn * 131 + B)
    assert np.array_equal(got, want)


# The at-scale configurations (batch 256 and 512 x both layouts x with and
# without the partial buffer, u64 keys, Zipf keys) at 2^24 keys, with the
# library's default wait limit of 2 s: no wait of a bulk insert or delete may
# come near it.
@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("pb", [True, False])
@pytest.mark.parametrize("B", [256, 512])
def test_heap_sort_2e24_default_wait_limit(variant, pb, B):
    got, want = run_heap_sort("u32", variant, pb, B, 1 << 24, seed=B + 24, chunk=B)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("key,dist,B", [("u64", "uniform", 1024), ("u32", "zipf", 2048), ("u64", "zipf", 512)])
def test_heap_sort_2e24_keys_and_zipf(variant, key, dist, B):
    got, want = run_heap_sort(key, variant, True, B, 1 << 24, dist=dist, seed=B + 7, chunk=B)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("B", [2048, 4096])
def test_heap_sort_large_batches(variant, B):
    got, want = run_heap_sort("u32", variant, True, B, 1 << 21, seed=B + 5)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("key", ["u64", "i32"])
@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
def test_heap_sort_key_types(key, variant):
    got, want = run_heap_sort(key, variant, True, 1024, 1 << 20, seed=3)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("dist", ["sorted", "reverse", "zipf"])
@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
def test_heap_sort_distributions(dist, variant):
    got, want = run_heap_sort("u32", variant, True, 1024, 1 << 20, dist=dist, seed=9)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("B", [256, 2048])
def test_heap_sort_ragged_sizes(B):
    """n not a multiple of the batch, inserts of odd sizes, partial buffer."""
    for n, chunk in [(1, 1), (B - 1, 7), (3 * B + 5, B), (10 * B + 17, B // 3 + 1)]:
        got, want = run_heap_sort("u32", "bottomup", True, B, n, seed=n, chunk=chunk)
        assert np.array_equal(got, want)
        got, want = run_heap_sort("u32", "topdown", True, B, n, seed=n + 1, chunk=chunk)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("B,chunk", [(256, 256), (256, 100), (1024, 333)])
def test_ragged_without_partial_buffer(variant, B, chunk):
    """Without the partial buffer a short insert is padded with init_limits
    and inserted as a full node; over many blocks every real key must come
    out, in order, followed by the padding (a padded node beside a node past
    the heap must not lose its keys)."""
    for n in (20 * B + 37, 9 * B + 1, 33 * B - 5):
        keys = pyoracle.gen("u32", n + chunk, "uniform", n)
        inserts = (n + chunk - 1) // chunk
        pad = inserts * B - n
        total = n + pad
        h = gh.Heap(batch_num_for(total, B), B, key="u32", variant=variant, partial_buffer=False)
        h.set_grid(16)
        h.insert(to_dev(keys, "u32"), chunk=chunk)
        assert h.item_count() == total
        out = empty_dev(total, "u32")
        for step in range(3):  # a few single deletes, then the rest in bulk
            assert h.delete_root(out) == B
        assert h.delete(out) == total - 3 * B  # the bulk delete writes from out[0]
        h.close()
        want = np.concatenate([np.sort(keys), np.full(pad, 0xFFFFFFFF, np.uint32)])
        got = to_host(out, "u32")
        assert np.array_equal(got[:total - 3 * B], want[3 * B:]), (n, chunk)


# test/heap_test.cu:120-171: insert half, concurrent insert + delete, delete the
# rest.  Deletes that overlap inserts need not come out in global order, so
# the bar is: no key lost or duplicated over the three phases, a valid heap
# after the concurrent phase, and a fully sorted final phase.
@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("pb", [True, False])
@pytest.mark.parametrize("B,logn", [(256, 20), (1024, 21)])
def test_concurrent_insert_and_delete(variant, pb, B, logn):
    n = 1 << logn
    for rep in range(3):
        keys = pyoracle.gen("u64", 77 + rep + B, "uniform", n)  # unique: (u32 << 32) | index
        h = gh.Heap(batch_num_for(n, B), B, key="u64", variant=variant, partial_buffer=pb)
        first, second = to_dev(keys[: n // 2], "u64"), to_dev(keys[n // 2:], "u64")
        h.insert(first, chunk=B)
        out1 = empty_dev(n, "u64")
        got1 = h.concurrent(second, out1, chunk=B if not pb else B // 2 + 3)
        ok, msg = h.check_insert_heap()
        assert ok, msg
        assert h.item_count() == n - got1
        out2 = empty_dev(n, "u64")
        got2 = h.delete(out2)
        assert got1 + got2 == n and h.is_empty()
        tail = to_host(out2, "u64")[:got2]
        assert np.all(tail[1:] >= tail[:-1])
        allout = np.concatenate([to_host(out1, "u64")[:got1], tail])
        assert np.array_equal(np.sort(allout), np.sort(keys))
        h.close()


def test_sort_entry_point():
    n, B = (1 << 20) + 333, 1024
    keys = pyoracle.gen("u32", 21, "uniform", n)
    h = gh.Heap(batch_num_for(n, B), B, key="u32", variant="bottomup")
    dk = to_dev(keys, "u32")
    out = empty_dev(n, "u32")
    for _ in range(2):
        h.sort(dk, out)
        assert np.array_equal(to_host(out, "u32"), np.sort(keys))
    h.close()


def test_empty_heap_and_output_limit():
    B = 256
    h = gh.Heap(64, B, key="u32", variant="topdown")
    out = empty_dev(4 * B, "u32")
    assert h.delete(out) == 0
    assert h.delete_root(out) == 0
    keys = pyoracle.gen("u32", 2, "uniform", 5 * B)
    h.insert(to_dev(keys, "u32"))
    # room for 2 batches only: stops before overflowing the output
    assert h.delete(out, max_keys=2 * B + 10) == 2 * B
    assert np.array_equal(to_host(out, "u32")[:2 * B], np.sort(keys)[:2 * B])
    assert h.item_count() == 3 * B
    h.close()


def expected_below(sorted_keys, B, t, pb):
    """Keys deleteRoot(.., app_t_val) takes from a heap of these keys: whole
    batches (the B smallest each time) while the smallest key is below t,
    then the partial buffer's remainder when only it is left."""
    n = len(sorted_keys)
    q, r = divmod(n, B) if pb else (n // B, 0)
    taken = 0
    for k in range(q):
        if not sorted_keys[k * B] < t:
            return taken
        taken += B
    if r and sorted_keys[q * B] < t:
        taken += r
    return taken


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("pb", [True, False])
@pytest.mark.parametrize("key,B", [("u32", 256), ("u64", 1024), ("i32", 512)])
def test_delete_below_threshold(variant, pb, key, B):
    """deleteRoot with app_t_val: deletes stop at the first batch whose
    smallest key is not below the threshold; the rest stays in the heap."""
    rng = np.random.default_rng(B)
    n = 40 * B + (B // 3 if pb else 0)
    keys = pyoracle.gen(key, B + len(key), "uniform", n)
    want = np.sort(keys)
    for frac in (0.0, 0.25, 0.5, 0.999, 1.0):
        idx = min(int(frac * n), n - 1)
        t = int(want[idx]) if frac < 1.0 else int(want[-1]) + 1
        if frac == 0.0:
            t = int(want[0])  # nothing is below the smallest key
        h = gh.Heap(batch_num_for(n, B), B, key=key, variant=variant, partial_buffer=pb)
        h.set_grid(int(rng.integers(1, 40)))
        h.insert(to_dev(keys, key), chunk=B // 3 if pb else B)
        out = empty_dev(n, key)
        got = h.delete_below(out, t)
        exp = expected_below(want, B, t, pb)
        assert got == exp, (frac, got, exp)
        assert np.array_equal(to_host(out, key)[:got], want[:got])
        assert h.item_count() == n - got
        ok, msg = h.check_insert_heap()
        assert ok, msg
        rest = empty_dev(n, key)
        assert h.delete(rest) == n - got
        assert np.array_equal(to_host(rest, key)[:n - got], want[got:])
        h.close()


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("pb", [True, False])
@pytest.mark.parametrize("key,B", [("u32", 256), ("u64", 512), ("i32", 1024)])
def test_gc_keeps_keys_below_threshold(variant, pb, key, B):
    """Device GC: after inserts and deletes, gc(t) keeps exactly the keys
    below t; the rebuilt heap passes checkInsertHeap and deletes them in
    order.  gc() with no threshold keeps every key."""
    n = 30 * B + (B // 5 if pb else 0)
    keys = pyoracle.gen(key, 7 * B, "uniform", n)
    h = gh.Heap(batch_num_for(n, B), B, key=key, variant=variant, partial_buffer=pb)
    h.set_grid(16)
    h.insert(to_dev(keys, key), chunk=B // 2 if pb else B)
    out = empty_dev(n, key)
    taken = h.delete(out, max_keys=5 * B)                  # a used heap: deletes moved the last nodes up
    assert taken == 5 * B
    left = np.sort(keys)[taken:]
    assert h.gc() == len(left)                            # keep everything
    ok, msg = h.check_insert_heap()
    assert ok, msg
    t = left[len(left) // 3] if key != "i32" else left[2 * len(left) // 3]
    kept = h.gc(int(t))
    want = left[left < t]
    assert kept == len(want)
    ok, msg = h.check_insert_heap()
    assert ok, msg
    pad = 0 if pb else (-kept) % B                          # the rebuild pads a short last insert
    assert h.item_count() == kept + pad
    got = h.delete(out)
    assert got == kept + pad
    assert np.array_equal(to_host(out, key)[:kept], want)
    h.close()


def test_gc_empty_and_all_dropped():
    B = 128
    h = gh.Heap(16, B, key="u32", variant="bottomup")
    assert h.gc(5) == 0
    keys = pyoracle.gen("u32", 3, "uniform", 4 * B + 7)
    h.insert(to_dev(keys, "u32"))
    assert h.gc(int(keys.min())) == 0                     # nothing is below the smallest key
    assert h.is_empty()
    ok, msg = h.check_insert_heap()
    assert ok, msg
    h.insert(to_dev(keys, "u32"))                         # the heap works after it
    out = empty_dev(len(keys), "u32")
    assert h.delete(out) == len(keys)
    assert np.array_equal(to_host(out, "u32"), np.sort(keys))
    h.close()


def test_capacity_error():
    B = 64
    h = gh.Heap(4, B, key="u32", variant="bottomup", partial_buffer=False)
    keys = to_dev(pyoracle.gen("u32", 4, "uniform", 6 * B), "u32")
    h.insert(keys, n=6 * B)
    with pytest.raises(gh.HeapError) as e:
        h.sync()
    assert e.value.status == gh.GH_ERR_CAPACITY
    h.reset()
    h.insert(keys, n=4 * B)
    h.sync()
    assert h.item_count() == 4 * B
    h.close()


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
def test_bounded_wait_reports_timeout(variant):
    """A lock word that nothing releases: the wait runs out, the kernel
    returns, the host reads GH_ERR_TIMEOUT and the heap works after reset."""
    B = 64
    h = gh.Heap(16, B, key="u32", variant=variant)
    h.set_timeout(0.05)
    keys = to_dev(pyoracle.gen("u32", 8, "uniform", B), "u32")
    h.inject_lock(0, 1)  # partial-buffer lock left taken
    h.insertion(keys, B)
    with pytest.raises(gh.HeapError) as e:
        h.sync()
    assert e.value.status == gh.GH_ERR_TIMEOUT
    items, status, counters = h.snapshot()
    assert counters[3] == gh.GH_ERR_TIMEOUT and counters[4] == 1  # partial-buffer lock site
    h.reset()
    h.insertion(keys, B)
    h.sync()
    assert h.item_count() == B
    h.close()


def test_invalid_arguments():
    with pytest.raises(gh.HeapError):
        gh.Heap(16, 100)  # not a power of two
    with pytest.raises(gh.HeapError):
        gh.Heap(16, 8)
    h = gh.Heap(16, 256)
    with pytest.raises(gh.HeapError):
        h.set_block_threads(48)
    with pytest.raises(gh.HeapError):
        h.set_timeout(61)  # above the 60 s bound of a wait
    with pytest.raises(gh.HeapError):
        h.set_timeout(0)
    with pytest.raises(gh.HeapError):
        h.insertion(empty_dev(512, "u32"), 300)  # size > batch_size
    h.close()


@pytest.mark.parametrize("key", ["u32", "u64", "i32"])
@pytest.mark.parametrize("dist", ["uniform", "sorted", "reverse", "zipf"])
def test_device_key_generator_matches_oracle(key, dist):
    """The benchmark's device-side workload generator (gh_gen_keys) makes the
    oracle's keys bit for bit."""
    n = (1 << 18) + 17
    got = to_host(gh.gen_keys(key, 1234, dist, n), key)
    assert np.array_equal(got, pyoracle.gen(key, 1234, dist, n))


@pytest.mark.parametrize("key,B,pb,n", [("u32", 2048, True, (1 << 22) + 777), ("u64", 1024, True, (1 << 20) + 5),
                                       ("i32", 512, False, 3000 * 512), ("u32", 256, True, 100)])
def test_sort_host_buffers(key, B, pb, n):
    """gh_heap_sort_host: pinned host keys in, host output in key order, the
    copies overlapped in pieces; repeated and with a larger n (the staging
    buffers grow); pageable numpy buffers work too."""
    dt = {"u32": torch.int32, "i32": torch.int32, "u64": torch.int64}[key]
    bn = 1
    while bn * B < 4 * n:
        bn <<= 1
    with gh.Heap(bn, B, key=key, partial_buffer=pb) as h:
        for m in (n // 2 // B * B or n, n):
            keys = gh.gen_keys(key, 31 + m, "uniform", m)
            want = gh.sort_keys(keys, key).cpu()
            hin = keys.cpu().pin_memory()
            hout = torch.empty(m, dtype=dt).pin_memory()
            h.sort_host(hin, hout)
            h.sync()
            assert torch.equal(hout, want)
        npin = keys.cpu().numpy().copy()
        npout = np.zeros_like(npin)
        h.sort_host(npin, npout)
        h.sync()
        assert np.array_equal(npout, want.numpy())
    if not pb:
        with gh.Heap(bn, B, key=key, partial_buffer=False) as h:
            with pytest.raises(Exception):
                h.sort_host(np.zeros(B + 1, np.int32), np.zeros(B + 1, np.int32))


@pytest.mark.parametrize("variant", ["bottomup", "topdown"])
def test_sort_with_more_blocks_than_the_gpu_holds(variant):
    """A grid of three blocks per SM: the reserved bulk insert and the
    owner-mode delete run at most the resident blocks (their blocks wait on
    each other), the result is exact and no wait runs out."""
    B, n = 2048, 1 << 22
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    keys = gh.gen_keys("u32", 71, "uniform", n)
    out = torch.empty_like(keys)
    with gh.Heap(4 * n // B, B, key="u32", variant=variant) as h:
        h.set_grid(3 * sms)
        h.sort(keys, out)
        h.sync()
        assert torch.equal(out, gh.sort_keys(keys, "u32"))
