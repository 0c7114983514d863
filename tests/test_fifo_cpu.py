"""CPU checks of the FIFO buffer: the sequential model of the reference's
Buffer<K> (oracle FifoModel), the multi-block checker, and the C ABI's
argument checks that answer without a GPU."""
import ctypes

import numpy as np
import pytest

from oracle import pyoracle


def test_model_positions_and_wrap():
    m = pyoracle.FifoModel(5)
    assert m.capacity == 8
    m.push(np.arange(7, dtype=np.uint32), 3)
    assert m.positions() == (0, 0, 7, 7)
    assert np.array_equal(m.pop(5, 2), np.arange(5))
    assert m.positions() == (5, 5, 7, 7)
    m.push(np.arange(100, 106, dtype=np.uint32), 4)   # wraps: slots 7, 0..4
    assert np.array_equal(m.pop(100, 4), np.array([5, 6, 100, 101, 102, 103, 104, 105]))
    assert m.positions() == (13, 13, 13, 13)
    assert len(m.pop(10, 3)) == 0


def test_model_full_ring():
    m = pyoracle.FifoModel(16)
    m.insert(np.arange(16, dtype=np.uint32))
    with pytest.raises(OverflowError):
        m.insert(np.arange(1, dtype=np.uint32))
    m.delete(1)
    m.insert(np.array([99], np.uint32))
    assert np.array_equal(m.pop(100, 16), np.r_[np.arange(1, 16), 99])


def test_reference_flow_sequential():
    """bufferTest.cu's check, sequentially: what comes out, sorted, is what went in."""
    n, block = 5000, 256
    keys = np.arange(2 * n, dtype=np.uint32)
    m = pyoracle.FifoModel(n)
    m.push(keys[:n], block)
    out = []
    for off in range(0, n, block):       # interleave: a third, the rest, one delete
        piece = keys[n + off:n + off + block]
        m.insert(piece[:len(piece) // 3])
        m.insert(piece[len(piece) // 3:])
        out.append(m.delete(min(block, n - off)))
    got = np.concatenate(out)
    assert np.array_equal(np.sort(got), keys[:n])
    assert np.array_equal(np.sort(m.pop(10 * n, block)), keys[n:])


def test_pieces_checker():
    inp = np.arange(10)
    starts = pyoracle.fifo_piece_starts(10, 4, False)
    assert list(starts) == [0, 4, 8]
    assert list(pyoracle.fifo_piece_starts(10, 4, True)) == [0, 1, 4, 5, 8]
    assert pyoracle.fifo_pieces_ok(inp, np.array([4, 5, 6, 7, 0, 1, 2, 3, 8, 9]), starts)
    assert not pyoracle.fifo_pieces_ok(inp, np.array([4, 5, 6, 7, 0, 1, 8, 9, 2, 3]), starts)  # piece split
    assert not pyoracle.fifo_pieces_ok(inp, np.array([1, 0, 2, 3, 4, 5, 6, 7, 8, 9]), starts)  # out of order
    assert not pyoracle.fifo_pieces_ok(inp, np.arange(1, 11), starts)                          # not a permutation


def test_capi_argument_checks(ghlib):
    import gpuheap_gb300 as gh
    vp = ctypes.c_void_p()
    assert ghlib.gh_fifo_create(None, 0, 16) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_create(ctypes.byref(vp), 7, 16) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_create(ctypes.byref(vp), 0, 0) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_create(ctypes.byref(vp), 0, (1 << 34) + 1) == gh.GH_ERR_INVALID
    assert not vp.value
    assert ghlib.gh_fifo_destroy(None) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_set_timeout(None, 1.0) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_set_launch(None, 0, 0) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_push(None, None, 0, 0, None) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_pop(None, None, 0, 0, None, None) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_concurrent(None, None, 0, 0, None, 0, None, None) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_inject_reservation(None, 1) == gh.GH_ERR_INVALID
    assert ghlib.gh_fifo_view_bytes() == 32
