"""The retrieving heap (gh_rheap_*): the heap of the reference's SSSP
application (applications/sssp_longfei_new/heap.cuh), whose retrieve()
takes the `size` smallest keys and refills the root in place.  Device code:
include/gpuheap_retrieve.cuh."""
import ctypes

import numpy as np

from . import _check, _I, _LL, _VP, lib

_KINDS = {"u32": (0, np.uint32, ctypes.c_uint32), "u64": (2, np.uint64, ctypes.c_uint64)}


def _ptr(t):
    return t.data_ptr() if hasattr(t, "data_ptr") else int(t)


def _stream(s):
    if s is None:
        return None
    return s.cuda_stream if hasattr(s, "cuda_stream") else s


class RetrievingHeap:
    """Heap<T>(batch_num, batch_size, init_limit) of the retrieving kind;
    key "u32" or "u64"; device buffers are torch tensors (or raw pointers)."""

    def __init__(self, batch_num, batch_size, key="u64", init_limit=None):
        kind, self.dtype, ctype = _KINDS[key]
        self.key, self.batch_num, self.batch_size = key, int(batch_num), int(batch_size)
        init = None if init_limit is None else ctypes.byref(ctype(int(init_limit)))
        h = _VP()
        _check(lib().gh_rheap_create(ctypes.byref(h), kind, self.batch_num, self.batch_size, init), "rheap_create")
        self._h = h

    def set_timeout(self, seconds):
        _check(lib().gh_rheap_set_timeout(self._h, float(seconds)), "rheap_set_timeout")

    def reset(self, stream=None):
        _check(lib().gh_rheap_reset(self._h, _stream(stream)), "rheap_reset")

    def insert(self, keys, count=None, stream=None):
        """insert(items, count): count (default: len(keys)) <= batch_size keys."""
        n = int(keys.numel() if count is None else count)
        _check(lib().gh_rheap_insert(self._h, _ptr(keys), n, _stream(stream)), "rheap_insert")

    def retrieve(self, out, size, stream=None):
        """retrieve(ret, *size): writes up to `size` smallest keys to out;
        returns how many."""
        sz = _I(int(size))
        _check(lib().gh_rheap_retrieve(self._h, _ptr(out), ctypes.byref(sz), _stream(stream)), "rheap_retrieve")
        return sz.value

    def concurrent(self, keys, chunk, inserters, retrievers, size, out, runs, stream=None):
        """One launch: inserters insert `keys` in chunks while retrievers
        retrieve `size` keys at a time; returns (keys out, runs)."""
        n_out, n_runs = _LL(), _I()
        _check(lib().gh_rheap_concurrent(self._h, _ptr(keys), int(keys.numel()), int(chunk), int(inserters),
                                         int(retrievers), int(size), _ptr(out), int(out.numel()), _ptr(runs),
                                         int(runs.numel()) // 2, ctypes.byref(n_out), ctypes.byref(n_runs),
                                         _stream(stream)), "rheap_concurrent")
        return n_out.value, n_runs.value

    def state(self):
        """(nodes, partial buffer, counters): numpy copies of every node and
        the partial buffer, counters = {batch_count, pb_size, error, steals,
        full, error_site}."""
        items = np.zeros(self.batch_num * self.batch_size, self.dtype)
        pb = np.zeros(self.batch_size, self.dtype)
        c = (_LL * 6)()
        _check(lib().gh_rheap_state(self._h, items.ctypes.data, pb.ctypes.data, c), "rheap_state")
        keys = ("batch_count", "pb_size", "error", "steals", "full", "error_site")
        return items, pb, {k: int(c[i]) for i, k in enumerate(keys)}

    def close(self):
        if getattr(self, "_h", None):
            lib().gh_rheap_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
