"""gh_heap_restore: a heap's snapshot, put back into the same heap after it
moved on or into a fresh heap of the same shape, resumes where the snapshot
left off -- same memory and counters, every lock word free, the checker
accepts the heap, and the remaining deletes give the sorted keys.  Kept in
a file of its own, collected last."""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402


def _drain_sorted(h, n):
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    assert h.delete(out) == n
    return out.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("variant", ["bottomup", "topdown"])
@pytest.mark.parametrize("pb", [True, False])
def test_restore_resumes_from_a_snapshot(ghlib, variant, pb):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    B = 64
    n = 20 * B + (37 if pb else 0)  # heaps without the partial buffer take full batches
    bn = 1
    while bn * B < 2 * n:
        bn <<= 1
    keys = pyoracle.gen("u32", 77, "uniform", n)
    want = np.sort(keys)
    dev = torch.from_numpy(keys.view(np.int32)).cuda()
    with gh.Heap(bn, B, key="u32", variant=variant, partial_buffer=pb) as h:
        h.insert(dev, n=n, chunk=B)
        h.sync()
        items, status, counters = h.snapshot()
        assert not status.any() and counters[3] == 0
        assert counters[0] * B + counters[1] == n

        assert np.array_equal(_drain_sorted(h, n), want)  # the heap moves on: empty now
        h.restore(items, counters)
        items2, status2, counters2 = h.snapshot()
        assert np.array_equal(items2, items)
        assert not status2.any()
        assert np.array_equal(counters2[:3], counters[:3]) and counters2[3] == 0
        ok, msg = h.check_insert_heap()
        assert ok, msg
        assert np.array_equal(_drain_sorted(h, n), want)

    with gh.Heap(bn, B, key="u32", variant=variant, partial_buffer=pb) as h2:
        h2.restore(items, counters)
        ok, msg = h2.check_insert_heap()
        assert ok, msg
        assert np.array_equal(_drain_sorted(h2, n), want)


def test_restore_refuses_counters_that_do_not_fit(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    with gh.Heap(8, 64, key="u32", variant="bottomup", partial_buffer=False) as h:
        items = np.full(9 * 64, 0xFFFFFFFF, np.uint32)
        for bad in ([9, 0, 0], [-1, 0, 0], [1, 5, 0], [1, 0, -3]):  # past batch_num; negative; pb without a buffer
            with pytest.raises(gh.HeapError):
                h.restore(items, bad)
        with pytest.raises(ValueError):
            h.restore(items[:-1], [0, 0, 0])
        h.restore(items, [0, 0, 0])
        items2, status2, counters2 = h.snapshot()
        assert np.array_equal(items2, items) and not status2.any() and not counters2[:4].any()
