"""retrieve() pinned to the reference's own retrieving heap
(applications/sssp_longfei_new/heap.cuh:79-270, run single-threaded on the
host by oracle/ref_retrieve_driver.cpp; vectors in
tests/golden/retrieve_ref_cases.npz, made by tests/golden/make_golden.py).

Every retrieve of the reference returned exactly the `size` smallest keys
held (fewer when fewer are held), ascending.  Checked here: the golden runs
against a sorted-multiset model (CPU), the project's oracle model of
`retrieve` -- delete the root batch, return the first `size`, insert the rest
back -- against the golden runs (CPU), and, where the reference's host build
exists, the reference itself against the vectors.  The GPU replay is in
test_retrieve_golden_gpu below (marked gpu).  Bar: bit-exact runs and counts.
The heaps' node contents are not compared: the reference's retrieving heap
is a different structure (0-based nodes, its partial buffer in an array of
its own, the root refilled in place from the partial buffer or the last
node), so its memory has no counterpart in this heap's."""
import bisect
import ctypes
import os

import numpy as np
import pytest

import golden_cases
from oracle import pyoracle

NP = {"u32": np.uint32, "u64": np.uint64}
IDS = range(len(golden_cases.retrieve_meta()))


def replay_multiset(c):
    ms, pos, runs, taken = [], 0, [], []
    for op in c["ops"]:
        if op > 0:
            for k in c["keys"][pos:pos + op]:
                bisect.insort(ms, int(k))
            pos += op
        else:
            t = min(-int(op), len(ms))
            runs.extend(ms[:t])
            taken.append(t)
            del ms[:t]
    return np.asarray(runs, NP[c["key"]]), np.asarray(taken, np.int32)


@pytest.mark.parametrize("i", IDS)
def test_golden_runs_are_the_smallest_keys(i):
    c = golden_cases.retrieve_case(i)
    runs, taken = replay_multiset(c)
    assert np.array_equal(taken, c["taken"]) and np.array_equal(runs, c["runs"])


def model_retrieve(m, size, B, dtype):
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
@pytest.mark.parametrize("i", IDS)
def test_oracle_model_returns_the_reference_runs(i, variant):
    c = golden_cases.retrieve_case(i)
    B = c["batch_size"]
    m = pyoracle.Model(c["key"], variant, True, 512, B)
    pos, runs, taken = 0, [], []
    for op in c["ops"]:
        if op > 0:
            assert m.insert(np.ascontiguousarray(c["keys"][pos:pos + op])) == 0
            pos += op
        else:
            got = model_retrieve(m, -int(op), B, NP[c["key"]])
            runs.append(got)
            taken.append(len(got))
    assert np.array_equal(np.asarray(taken, np.int32), c["taken"])
    assert np.array_equal(np.concatenate(runs), c["runs"])


@pytest.mark.parametrize("i", IDS)
def test_reference_host_run_reproduces_the_vectors(i):
    lib_path = os.path.join(os.path.dirname(pyoracle.HERE), "oracle", "_ref", "libbgpq_ref.so")
    if not os.path.exists(lib_path):
        pytest.skip("reference heaps not built here (set GH_REFERENCE_TREE for build())")
    ref = ctypes.CDLL(lib_path)
    c = golden_cases.retrieve_case(i)
    kind, B = c["key"], c["batch_size"]

    def f(name, res=ctypes.c_int):
        fn = getattr(ref, f"rr_{kind}_{name}")
        fn.restype = res
        return fn

    create = f("create", ctypes.c_void_p)
    create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint32 if kind == "u32" else ctypes.c_uint64]
    h = create(512, B, 0xFFFFFFFF if kind == "u32" else 2**64 - 1)
    pos, runs, taken = 0, [], []
    for op in c["ops"]:
        if op > 0:
            chunk = np.ascontiguousarray(c["keys"][pos:pos + op])
            assert f("insert")(ctypes.c_void_p(h), ctypes.c_void_p(chunk.ctypes.data), int(op)) == 0
            pos += op
        else:
            out = np.zeros(B, NP[kind])
            sz = ctypes.c_int(-int(op))
            assert f("retrieve")(ctypes.c_void_p(h), ctypes.c_void_p(out.ctypes.data), ctypes.byref(sz)) == 0
            runs.append(out[:sz.value].copy())
            taken.append(sz.value)
    f("destroy", None)(ctypes.c_void_p(h))
    assert np.array_equal(np.asarray(taken, np.int32), c["taken"])
    assert np.array_equal(np.concatenate(runs), c["runs"])


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["topdown", "bottomup"])
@pytest.mark.parametrize("i", IDS)
def test_retrieve_golden_gpu(i, variant, ghlib):
    """One block replays the sequence through gh_heap_insert_batch and
    gh_heap_retrieve: every run equals the reference's, bit for bit."""
    torch = pytest.importorskip("torch")
    import gpuheap_gb300 as gh
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = golden_cases.retrieve_case(i)
    kind, B = c["key"], c["batch_size"]
    store = np.int32 if kind == "u32" else np.int64
    keys = torch.from_numpy(np.ascontiguousarray(c["keys"]).view(store)).cuda()
    out = torch.zeros(B, dtype=torch.int32 if kind == "u32" else torch.int64, device="cuda")
    pos, runs, taken = 0, [], []
    with gh.Heap(512, B, key=kind, variant=variant, partial_buffer=True) as h:
        for op in c["ops"]:
            if op > 0:
                h.insertion(keys[pos:pos + int(op)], int(op))
                pos += int(op)
            else:
                got = h.retrieve(out, -int(op))
                runs.append(out.cpu().numpy().view(NP[kind])[:got].copy())
                taken.append(got)
    assert np.array_equal(np.asarray(taken, np.int32), c["taken"])
    assert np.array_equal(np.concatenate(runs), c["runs"])
