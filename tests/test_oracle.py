"""CPU tests of the oracle: pinned against the reference's own heap code
(golden vectors), the checker against planted mistakes, the generators and
the algorithmic byte model."""
import numpy as np
import pytest

import golden_cases
from oracle import pyoracle

GOLDEN = golden_cases.all_ids()


def replay_model(c):
    """Runs a golden case's operation list through the oracle model."""
    variant = "topdown" if c["topdown"] else "bottomup"
    m = pyoracle.Model(c["key"], variant, c["partial_buffer"], c["batch_num"], c["batch_size"])
    keys = c["keys"]
    out = np.zeros_like(c["out"])
    pos, dsizes, snap = 0, [], None
    for op in c["ops"]:
        if op > 0:
            assert m.insert(keys[pos:pos + op]) == 0
            pos += op
        elif op == 0:
            dsizes.append(m.delete(out))
        else:
            snap = m.state()
    items, counters = m.state()
    return out, np.asarray(dsizes, np.int32), snap, items, counters


@pytest.mark.parametrize("which,i", GOLDEN)
def test_model_matches_reference_golden(which, i):
    c = golden_cases.case(i, which)
    out, dsizes, snap, items, counters = replay_model(c)
    assert np.array_equal(dsizes, c["dsizes"]), "deleteRoot sizes"
    assert np.array_equal(out, c["out"]), "HEAP_SORT output stream"
    assert np.array_equal(snap[0], c["snap_items"]), "heap memory after the insert phase"
    assert np.array_equal(snap[1], c["snap_counters"]), "counters after the insert phase"
    assert np.array_equal(items, c["items"]), "final heap memory"
    assert np.array_equal(counters, c["counters"]), "final counters"


@pytest.mark.parametrize("which,i", GOLDEN)
def test_golden_is_a_priority_queue(which, i):
    """Every deleteRoot of the reference run output the smallest keys present
    at that moment; a pure insert-then-drain run is std::sort of the input
    (test/heap_test.cu:163-170)."""
    c = golden_cases.case(i, which)
    keys, out = c["keys"], c["out"]
    present = np.empty(0, keys.dtype)
    pos = cursor = d = 0
    for op in c["ops"]:
        if op > 0:
            present = np.sort(np.concatenate([present, keys[pos:pos + op]]))
            pos += op
        elif op == 0:
            sz = int(c["dsizes"][d])
            d += 1
            assert np.array_equal(out[cursor:cursor + sz], present[:sz])
            present = present[sz:]
            cursor += sz
    assert present.size == 0 and cursor == c["n"]
    if c["scenario"] == "sort":
        assert np.array_equal(out[:c["n"]], np.sort(keys))


def _case_index(variant, key, scenario):
    return next(m["case"] for m in golden_cases.meta()
                if (m["variant"], m["key"], m["scenario"]) == (variant, key, scenario))


# distinct keys and at least three full nodes: not the "ties" cases
@pytest.mark.parametrize("which", [("tditdd", "u32", "sort"), ("tditdd", "i32", "concurrent"),
                                   ("buitdd", "u32", "concurrent"), ("buitdd_np", "u64", "sort")])
def test_checker_accepts_golden_snapshot_and_catches_planted_mistakes(which):
    c = golden_cases.case(_case_index(*which))
    variant = "topdown" if c["topdown"] else "bottomup"
    B = c["batch_size"]
    items = c["snap_items"].copy()
    bc, ps = int(c["snap_counters"][0]), int(c["snap_counters"][1])
    status = np.zeros(c["batch_num"] + 1, np.int32)
    assert pyoracle.check_heap(variant, items, status, B, bc, ps)
    assert bc >= 3
    # unsorted node
    bad = items.copy()
    bad[2 * B], bad[2 * B + 1] = bad[2 * B + 1], bad[2 * B]
    if bad[2 * B] != bad[2 * B + 1]:
        r = pyoracle.check_heap(variant, bad, status, B, bc, ps)
        assert not r and "unsorted" in r[1]
    # child starting below its parent's last key
    # (node 3's parent is the root in both layouts; lowering its first key keeps it sorted)
    bad = items.copy()
    bad[3 * B] = bad[2 * B - 1] - 1
    r = pyoracle.check_heap(variant, bad, status, B, bc, ps)
    assert not r and "parent" in r[1]
    # a lock word left taken
    st = status.copy()
    st[bc] = 1
    r = pyoracle.check_heap(variant, items, st, B, bc, ps)
    assert not r and "state" in r[1]


def test_checker_partial_buffer_below_root():
    B = 16
    items = np.full(4 * B, 2**32 - 1, np.uint32)
    items[B:2 * B] = np.arange(100, 100 + B)          # root
    items[0:3] = [50, 60, 70]                          # partial buffer below the root
    status = np.zeros(4, np.int32)
    r = pyoracle.check_heap("bottomup", items, status, B, 1, 3)
    assert not r and "partial" in r[1]
    items[0:3] = [200, 210, 220]
    assert pyoracle.check_heap("bottomup", items, status, B, 1, 3)


def test_reversed_index_matches_reference_formula():
    # heap/buitdd/heap.cuh:233-236 on the GPU: (brev(i) >> (clz(i)+1)) | (1 << (31-clz(i)))
    def ref(i):
        if i == 1:
            return 1
        clz = 32 - i.bit_length()
        l = clz + 1
        b = int(format(i, "032b")[::-1], 2)
        return (b >> l) | (1 << (32 - l))
    for i in range(1, 5000):
        assert pyoracle.reversed_idx(i) == ref(i)
        assert pyoracle.reversed_idx(pyoracle.reversed_idx(i)) == i


@pytest.mark.parametrize("key", ["u32", "u64", "i32"])
@pytest.mark.parametrize("dist", ["uniform", "sorted", "reverse", "zipf"])
def test_generators(key, dist):
    n = 1 << 16
    a = pyoracle.gen(key, 11, dist, n)
    b = pyoracle.gen(key, 11, dist, n, threads=1)
    assert np.array_equal(a, b), "deterministic for any thread count"
    assert not np.array_equal(a, pyoracle.gen(key, 12, dist, n))
    init = pyoracle.INIT[key]
    assert int(a.max()) < init
    if dist == "sorted":
        assert np.all(np.diff(a.astype(np.float64)) >= 0)
    if dist == "reverse":
        assert np.all(np.diff(a.astype(np.float64)) <= 0)
    if key == "u64":
        payload = (a & np.uint64(0xFFFFFFFF)).astype(np.int64)
        assert np.array_equal(np.sort(payload), np.arange(n)), "payload is the input index"
    if dist == "zipf":
        hi = (a >> np.uint64(32)) if key == "u64" else a
        vals, counts = np.unique(hi, return_counts=True)
        assert len(vals) <= 1 << 16
        # rank-1 share of Zipf(1.2) over 2^16 values is 1/H where H = sum r^-1.2
        h = np.sum(np.arange(1, (1 << 16) + 1, dtype=np.float64) ** -1.2)
        assert abs(counts.max() / n - 1.0 / h) < 0.01


def test_uniform_covers_range():
    a = pyoracle.gen("u32", 3, "uniform", 1 << 20)
    assert a.min() < 2**24 and a.max() > 2**32 - 2**24


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_parallel_sort(threads):
    a = pyoracle.gen("u32", 5, "uniform", (1 << 20) + 7)
    want = np.sort(a)
    pyoracle.sort(a, threads=threads)
    assert np.array_equal(a, want)


@pytest.mark.parametrize("n,B,s,pb,per_key", [
    (2**20, 1024, 4, True, 196.2), (2**28, 256, 4, True, 396.0), (2**28, 1024, 4, True, 356.0),
    (2**28, 1024, 4, False, 340.0), (2**28, 2048, 4, True, 336.0), (2**28, 1024, 8, True, 712.0)])
def test_sort_bytes_model(n, B, s, pb, per_key):
    assert abs(pyoracle.sort_bytes(n, B, s, pb) / n - per_key) < 0.1


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("pb", [True, False])
def test_model_heap_sort_random(variant, pb):
    rng = np.random.default_rng(5)
    B = 64
    n = 300 * B
    keys = rng.integers(0, 2**32 - 1, n, dtype=np.uint32)
    m = pyoracle.Model("u32", variant, pb, 1024, B)
    step = B // 3 if pb else B
    for p in range(0, n, step):
        assert m.insert(keys[p:p + step]) == 0
    items, counters = m.state()
    assert pyoracle.check_heap(variant, items, None, B, counters[0], counters[1])
    out = np.zeros(n + B, np.uint32)
    while m.delete(out):
        pass
    assert np.array_equal(out[:n], np.sort(keys))


def padded_sequence(seed, B=16):
    """Full inserts of B keys plus one short insert at a random place: without
    the partial buffer the short one is padded with init_limits and inserted
    as a full node."""
    rng = np.random.default_rng(seed)
    nfull = int(rng.integers(3, 12))
    tail = int(rng.integers(1, B))
    keys = rng.integers(0, 2**32 - 1, nfull * B + tail, dtype=np.uint32)
    pieces = [B] * nfull
    pieces.insert(int(rng.integers(0, nfull + 1)), tail)
    return keys, pieces, B - tail


@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
def test_model_keeps_padded_keys(variant):
    """A padded node whose sibling lies past the heap (all init_limits) ties
    with it on the last key.  The larger child is then the one with the larger
    first key, so the carried batch -- with the padded node's real keys --
    stays inside the heap; every key comes out, in order."""
    B = 16
    for seed in range(200):
        keys, pieces, pad = padded_sequence(seed, B)
        m = pyoracle.Model("u32", variant, False, 1024, B)
        pos = 0
        for p in pieces:
            assert m.insert(keys[pos:pos + p]) == 0
            pos += p
        out = np.zeros(len(keys) + pad + 4 * B, np.uint32)
        while m.delete(out):
            pass
        want = np.concatenate([np.sort(keys), np.full(pad, 0xFFFFFFFF, np.uint32)])
        assert np.array_equal(out[:len(want)], want), seed


def test_reference_loses_padded_keys():
    """The reference's tie rule (tditdd_np/heap.cuh:416: the left child on a
    tie) loses the real keys of a padded node in the sequence below; the
    model keeps them.  The host run is deterministic: every call of the
    reference starts from a cleared shared-memory stand-in and spin counter
    (oracle/ref_driver.cpp), and on this sequence its sift reads lock words
    past the end of its status array (tditdd_np/heap.cuh:356), which land in
    the room the shim's allocations keep behind them, filled with a value it
    takes as "no child" (oracle/ref_shim.h).  Before that room existed those
    reads saw whatever the host heap held, and about one full test run in six
    stopped here.  Runs only where oracle/_ref holds the reference's heaps
    compiled for the host (built from the reference tree)."""
    import ctypes
    import os
    lib_path = os.path.join(os.path.dirname(pyoracle.HERE), "oracle", "_ref", "libbgpq_ref.so")
    if not os.path.exists(lib_path):
        pytest.skip("reference heaps not built here")
    ref = ctypes.CDLL(lib_path)
    vp = ctypes.c_void_p

    def fn(name, res=ctypes.c_int):
        f = getattr(ref, f"tditdd_np_u32_{name}")
        f.restype = res
        return f

    keys, pieces, pad = padded_sequence(28)
    B = 16
    create = fn("create", vp)
    create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32]
    h = create(1024, B, 0xFFFFFFFF)
    m = pyoracle.Model("u32", "topdown", False, 1024, B)
    pos = 0
    for p in pieces:
        chunk = np.ascontiguousarray(keys[pos:pos + p])
        pos += p
        assert fn("insert")(vp(h), vp(chunk.ctypes.data), p) == 0
        assert m.insert(chunk) == 0
    n_out = len(keys) + pad
    ref_out = np.zeros(n_out + 4 * B, np.uint32)
    model_out = np.zeros(n_out + 4 * B, np.uint32)
    sz = ctypes.c_int()
    for _ in range(len(pieces) + 2):
        m.delete(model_out)
        assert fn("delete")(vp(h), vp(ref_out.ctypes.data), ctypes.byref(sz)) == 0, "the host run stopped"
    fn("destroy", None)(vp(h))
    want = np.concatenate([np.sort(keys), np.full(pad, 0xFFFFFFFF, np.uint32)])
    assert np.array_equal(model_out[:n_out], want)
    assert not np.array_equal(np.sort(ref_out[:n_out]), want), "the reference kept every key here"


def test_model_capacity():
    m = pyoracle.Model("u32", "topdown", False, 2, 16)
    k = np.arange(16, dtype=np.uint32)
    assert m.insert(k) == 0 and m.insert(k) == 0
    assert m.insert(k) == -2
