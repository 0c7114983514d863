"""gh_sort_noalloc: the heap-sort for callers that cannot allocate device
memory when they sort (a framework's caching allocator already holds the GPU,
or a latency-critical path that cannot take cudaMalloc's implicit device
synchronization).  Its heap lives in a fixed device array of the library, so
this checks it through the C ABI against gh_heap_sort on the same inputs, two
calls in a row (the array keeps the previous call's contents), for every key
type with and without the partial buffer, and that sizes beyond the array
(or a ragged size without the partial buffer) are refused.  Kept in a file of
its own, collected last."""
import ctypes

import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402

GH_OK, GH_ERR_INVALID, GH_ERR_CAPACITY = 0, 1, 2
KIND = {"u32": 0, "i32": 1, "u64": 2}
VIEW = {"u32": (np.int32, np.uint32), "i32": (np.int32, np.int32), "u64": (np.int64, np.uint64)}


def _sorted_by_existing_entry_point(dev_in, n, B, key, variant, pb):
    bn = 1
    while bn * B < 2 * n:
        bn <<= 1
    out = torch.empty_like(dev_in)
    with gh.Heap(bn, B, key=key, variant=variant, partial_buffer=pb) as h:
        h.sort(dev_in, out, n=n)
    return out


@pytest.fixture(autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)


@pytest.mark.parametrize("variant", ["bottomup", "topdown"])
def test_noalloc_sort_matches_heap_sort_twice(ghlib, variant):
    vcode = 1 if variant == "bottomup" else 0
    for call, (n, B) in enumerate([((1 << 20) + 333, 1024), (777_777, 512)]):
        keys = pyoracle.gen("u32", 500 + call, "uniform", n)
        dev_in = torch.from_numpy(keys.view(np.int32)).cuda()
        want = _sorted_by_existing_entry_point(dev_in, n, B, "u32", variant, True)
        got = torch.full_like(dev_in, -1)
        st = ghlib.gh_sort_noalloc(0, vcode, 1, B, ctypes.c_void_p(dev_in.data_ptr()), n,
                                   ctypes.c_void_p(got.data_ptr()), None)
        assert st == GH_OK, gh.lib().gh_status_string(st)
        assert torch.equal(got, want), f"call {call}: differs from gh_heap_sort"
        assert np.array_equal(got.cpu().numpy().view(np.uint32), np.sort(keys))


@pytest.mark.parametrize("key", ["u32", "i32", "u64"])
@pytest.mark.parametrize("pb", [1, 0])
def test_noalloc_key_types_and_partial_buffer(ghlib, key, pb):
    """Each key type (the i32 branch with its own padding key, the 8-byte
    keys with their own size limit), with and without the partial buffer:
    two calls in a row equal gh_heap_sort and np.sort."""
    B = 256
    store, npk = VIEW[key]
    for call, n in enumerate([3 * B + 17 if pb else 3 * B, 40 * B + (5 if pb else 0)]):
        keys = pyoracle.gen(key, 900 + call + 10 * pb, "uniform", n)
        dev_in = torch.from_numpy(keys.view(store)).cuda()
        want = _sorted_by_existing_entry_point(dev_in, n, B, key, "bottomup", bool(pb))
        got = torch.full_like(dev_in, -1)
        st = ghlib.gh_sort_noalloc(KIND[key], 1, pb, B, ctypes.c_void_p(dev_in.data_ptr()), n,
                                   ctypes.c_void_p(got.data_ptr()), None)
        assert st == GH_OK, gh.lib().gh_status_string(st)
        assert torch.equal(got, want), f"{key} pb={pb} call {call}: differs from gh_heap_sort"
        assert np.array_equal(got.cpu().numpy().view(npk), np.sort(keys))


def test_noalloc_rejects_sizes_beyond_its_array(ghlib):
    n = 8 << 20  # 32 MiB of u32 keys alone: cannot fit the 16 MiB array
    dev_in = torch.zeros(16, dtype=torch.int32, device="cuda")
    st = ghlib.gh_sort_noalloc(0, 1, 1, 1024, ctypes.c_void_p(dev_in.data_ptr()), n,
                               ctypes.c_void_p(dev_in.data_ptr()), None)
    assert st == GH_ERR_CAPACITY
    # without the partial buffer only whole batches: a ragged n is refused up front
    st = ghlib.gh_sort_noalloc(0, 1, 0, 256, ctypes.c_void_p(dev_in.data_ptr()), 3 * 256 + 1,
                               ctypes.c_void_p(dev_in.data_ptr()), None)
    assert st == GH_ERR_INVALID
