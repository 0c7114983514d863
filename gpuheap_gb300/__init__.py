"""gpuheap_gb300: a GB300-native batched priority queue (BGPQ).

Host-side mirror of the reference's `Heap<K>` (ruadapt/gpuheap,
heap/{tditdd,tditdd_np,buitdd,buitdd_np}/heap.cuh) over the C ABI of
libgpuheap_gb300.so (include/gpuheap.h).  Device buffers are torch CUDA
tensors (or anything with .data_ptr()); torch is only plumbing here.

The reference picks the variant by include path; here it is an argument:
    variant="topdown"  + partial_buffer=True   == tditdd
    variant="topdown"  + partial_buffer=False  == tditdd_np
    variant="bottomup" + partial_buffer=True   == buitdd
    variant="bottomup" + partial_buffer=False  == buitdd_np

The library is required: importing works without it, but every call raises
if libgpuheap_gb300.so cannot be loaded (there is no CPU fallback).
"""
import ctypes
import os

__all__ = ["Heap", "HeapError", "KEY_KINDS", "lib", "library_path", "build"]

_HERE = os.path.dirname(os.path.abspath(__file__))
library_path = os.path.join(_HERE, "libgpuheap_gb300.so")

KEY_KINDS = {"u32": 0, "i32": 1, "u64": 2}
_KEY_BYTES = {"u32": 4, "i32": 4, "u64": 8}
_KEY_CTYPE = {"u32": ctypes.c_uint32, "i32": ctypes.c_int32, "u64": ctypes.c_uint64}
_VARIANTS = {"topdown": 0, "td": 0, "bottomup": 1, "bu": 1}

GH_OK, GH_ERR_INVALID, GH_ERR_CAPACITY, GH_ERR_TIMEOUT, GH_ERR_CUDA, GH_ERR_STATE = range(6)

_VP = ctypes.c_void_p
_I = ctypes.c_int
_LL = ctypes.c_longlong
_SIGS = {
    "gh_status_string": (ctypes.c_char_p, [_I]),
    "gh_heap_create": (_I, [ctypes.POINTER(_VP), _I, _I, _I, _I, _I, _VP]),
    "gh_heap_destroy": (_I, [_VP]),
    "gh_heap_reset": (_I, [_VP, _VP]),
    "gh_heap_set_timeout": (_I, [_VP, ctypes.c_double]),
    "gh_heap_set_block_threads": (_I, [_VP, _I]),
    "gh_heap_set_grid": (_I, [_VP, _I]),
    "gh_heap_set_owner_depth": (_I, [_VP, _I]),
    "gh_heap_insert": (_I, [_VP, _VP, _LL, _I, _VP]),
    "gh_heap_delete": (_I, [_VP, _VP, _LL, ctypes.POINTER(_LL), _VP]),
    "gh_heap_delete_below": (_I, [_VP, _VP, _LL, _VP, ctypes.POINTER(_LL), _VP]),
    "gh_heap_gc": (_I, [_VP, _VP, ctypes.POINTER(_LL), _VP]),
    "gh_heap_concurrent": (_I, [_VP, _VP, _LL, _I, _VP, _LL, ctypes.POINTER(_LL), _VP]),
    "gh_heap_sync": (_I, [_VP, _VP]),
    "gh_heap_insert_batch": (_I, [_VP, _VP, _I, _VP]),
    "gh_heap_delete_batch": (_I, [_VP, _VP, ctypes.POINTER(_I), _VP]),
    "gh_heap_retrieve": (_I, [_VP, _VP, _I, ctypes.POINTER(_I), _VP]),
    "gh_heap_sort": (_I, [_VP, _VP, _LL, _VP, _VP]),
    "gh_heap_sort_host": (_I, [_VP, _VP, _LL, _VP, _VP]),
    "gh_heap_check": (_I, [_VP, ctypes.POINTER(_I), ctypes.c_char_p, _I, _VP]),
    "gh_heap_item_count": (_I, [_VP, ctypes.POINTER(_LL)]),
    "gh_heap_node_count": (_I, [_VP, ctypes.POINTER(_I)]),
    "gh_heap_is_empty": (_I, [_VP, ctypes.POINTER(_I)]),
    "gh_heap_snapshot": (_I, [_VP, _VP, _VP, _VP]),
    "gh_heap_restore": (_I, [_VP, _VP, _VP]),
    "gh_heap_inject_lock": (_I, [_VP, _I, _I]),
    "gh_launch_count": (_LL, []),
    "gh_heap_owner_stats": (_I, [_VP, _VP, _I]),
    "gh_merge_batches": (_I, [_I, _I, _VP, _VP, _I, _VP, _VP, _I, _VP]),
    "gh_sort_batch": (_I, [_I, _VP, _I, _VP, _I, _VP]),
    "gh_sort_noalloc": (_I, [_I, _I, _I, _I, _VP, _LL, _VP, _VP]),
    "gh_gen_keys": (_I, [_I, _I, ctypes.c_ulonglong, _LL, _VP, _VP]),
    "gh_rmat_edges": (_I, [_I, _LL, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_ulonglong,
                           ctypes.c_uint, _VP, _VP, _VP, _VP]),
    "gh_sssp": (_I, [_VP, _I, _VP, _VP, _VP, _I, _VP, _VP, ctypes.POINTER(ctypes.c_ulonglong)]),
    "gh_rheap_create": (_I, [ctypes.POINTER(_VP), _I, _I, _I, _VP]),
    "gh_rheap_destroy": (_I, [_VP]),
    "gh_rheap_reset": (_I, [_VP, _VP]),
    "gh_rheap_set_timeout": (_I, [_VP, ctypes.c_double]),
    "gh_rheap_insert": (_I, [_VP, _VP, _I, _VP]),
    "gh_rheap_retrieve": (_I, [_VP, _VP, ctypes.POINTER(_I), _VP]),
    "gh_rheap_concurrent": (_I, [_VP, _VP, _LL, _I, _I, _I, _I, _VP, _LL, _VP, _I, ctypes.POINTER(_LL),
                                 ctypes.POINTER(_I), _VP]),
    "gh_rheap_state": (_I, [_VP, _VP, _VP, _VP]),
    "gh_sssp_retrieve": (_I, [_I, _VP, _VP, _VP, _I, _VP, _I, _I, _I, _LL, _VP, ctypes.POINTER(ctypes.c_ulonglong)]),
    "gh_heap_view_bytes": (ctypes.c_size_t, []),
    "gh_heap_device_view": (_I, [_VP, _VP, ctypes.c_size_t]),
    "gh_heap_smem_bytes": (ctypes.c_size_t, [_I, _I]),
    "gh_heap_info": (_I, [_VP] + [ctypes.POINTER(_I)] * 7),
    "gh_batch_create": (_I, [ctypes.POINTER(_VP), _I, _I, _I]),
    "gh_batch_destroy": (_I, [_VP]),
    "gh_batch_set_timeout": (_I, [_VP, ctypes.c_double]),
    "gh_batch_set_astar_blocks": (_I, [_VP, _LL, _I]),
    "gh_batch_set_knapsack_order": (_I, [_VP, _I, _I]),
    "gh_batch_knapsack_switches": (_I, [_VP, _VP, _VP]),
    "gh_batch_add_astar": (_I, [_VP, _I, _I, _VP, ctypes.POINTER(_I)]),
    "gh_batch_add_astar_bitmap": (_I, [_VP, _I, _I, _VP, ctypes.POINTER(_I)]),
    "gh_batch_add_knapsack": (_I, [_VP, _I, _VP, _VP, _LL, ctypes.POINTER(_I)]),
    "gh_batch_build": (_I, [_VP, _VP]),
    "gh_batch_run": (_I, [_VP, _I, _VP]),
    "gh_batch_plain_times": (_I, [_VP, _VP]),
    "gh_batch_results": (_I, [_VP, _VP, _VP, _VP, _VP]),
    "gh_batch_info": (_I, [_VP, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                           ctypes.POINTER(_LL)]),
    "gh_gen_grid": (_I, [_I, _I, ctypes.c_ulonglong, _I, _VP, _I]),
    "gh_serve_create": (_I, [ctypes.POINTER(_VP), _LL, _I, _I, _I, _I]),
    "gh_serve_destroy": (_I, [_VP]),
    "gh_serve_set_blocks": (_I, [_VP, _LL, _I, _LL, _I]),
    "gh_serve_add_graph": (_I, [_VP, _I, _VP, _VP, _VP, ctypes.POINTER(_I)]),
    "gh_serve_add_map": (_I, [_VP, _I, _I, _VP, ctypes.POINTER(_I)]),
    "gh_serve_add_bitmap": (_I, [_VP, _I, _I, _VP, ctypes.POINTER(_I)]),
    "gh_serve_submit": (_I, [_VP, _I, _I, _I, _I, ctypes.POINTER(_LL)]),
    "gh_serve_step": (_I, [_VP, _VP, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "gh_serve_result": (_I, [_VP, _LL, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_ulonglong),
                             ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(_LL)]),
    "gh_serve_finished": (_I, [_VP, _VP, _I, ctypes.POINTER(_I)]),
    "gh_serve_info": (_I, [_VP, ctypes.POINTER(_LL), ctypes.POINTER(_LL), ctypes.POINTER(_I), ctypes.POINTER(_LL)]),
    "gh_serve_start": (_I, [_VP, _I]),
    "gh_serve_poll": (_I, [_VP, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "gh_serve_stop": (_I, [_VP]),
    "gh_fifo_create": (_I, [ctypes.POINTER(_VP), _I, _LL]),
    "gh_fifo_destroy": (_I, [_VP]),
    "gh_fifo_reset": (_I, [_VP, _VP]),
    "gh_fifo_set_timeout": (_I, [_VP, ctypes.c_double]),
    "gh_fifo_set_launch": (_I, [_VP, _I, _I]),
    "gh_fifo_push": (_I, [_VP, _VP, _LL, _I, _VP]),
    "gh_fifo_pop": (_I, [_VP, _VP, _LL, _I, ctypes.POINTER(_LL), _VP]),
    "gh_fifo_concurrent": (_I, [_VP, _VP, _LL, _I, _VP, _LL, ctypes.POINTER(_LL), _VP]),
    "gh_fifo_count": (_I, [_VP, ctypes.POINTER(_LL)]),
    "gh_fifo_positions": (_I, [_VP] + [ctypes.POINTER(ctypes.c_ulonglong)] * 4),
    "gh_fifo_snapshot": (_I, [_VP, _VP, _VP]),
    "gh_fifo_view_bytes": (ctypes.c_size_t, []),
    "gh_fifo_device_view": (_I, [_VP, _VP, ctypes.c_size_t]),
    "gh_fifo_inject_reservation": (_I, [_VP, _LL]),
    "gh_fifo_info": (_I, [_VP, ctypes.POINTER(_I), ctypes.POINTER(_LL), ctypes.POINTER(_I), ctypes.POINTER(_I),
                          ctypes.POINTER(_I)]),
}

_lib = None


def build(verbose=False):
    """Compiles the CUDA library in-tree (gpuheap_gb300/builder.py)."""
    from . import builder
    return builder.build(verbose=verbose)


def lib():
    """The loaded C ABI library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(library_path):
            raise RuntimeError(
                f"gpuheap_gb300: {library_path} is missing; build it with "
                "`python -c 'import gpuheap_gb300 as g; g.build()'`")
        so = ctypes.CDLL(library_path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(so, name)
            fn.restype = res
            fn.argtypes = args
        _lib = so
    return _lib


def gen_keys(key, seed, dist, n, device="cuda"):
    """Seeded keys of the plain heap-sort workload on the device (gh_gen_keys):
    uniform / zipf made there; sorted and reverse are uniform keys sorted in
    key order.  Returns a torch tensor of the key's width (int32 / int64 bits)."""
    import torch
    dt = torch.int64 if key == "u64" else torch.int32
    out = torch.empty(int(n), dtype=dt, device=device)
    st = lib().gh_gen_keys(KEY_KINDS[key], 1 if dist == "zipf" else 0, int(seed), int(n), out.data_ptr(),
                           torch.cuda.current_stream().cuda_stream)
    _check(st, "gen_keys")
    if dist in ("sorted", "reverse"):
        out = sort_keys(out, key)
        if dist == "reverse":
            out = out.flip(0)
    elif dist not in ("uniform", "zipf"):
        raise ValueError(f"unknown distribution {dist}")
    return out


def sort_keys(t, key):
    """Key-order sort of a tensor holding key bits (torch; for checks and inputs)."""
    import torch
    if key == "i32":
        return torch.sort(t).values
    if key == "u32":
        return torch.sort(t.to(torch.int64) & 0xFFFFFFFF).values.to(torch.int32)
    flip = torch.tensor(-(2**63), dtype=torch.int64, device=t.device)
    return torch.sort(t ^ flip).values ^ flip


def launch_count():
    """Kernels launched by libgpuheap_gb300.so so far."""
    return lib().gh_launch_count()


class HeapError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = lib().gh_status_string(status).decode()
        super().__init__(f"{where}: {msg} (status {status})")


def _check(status, where):
    if status != GH_OK:
        raise HeapError(status, where)


def _ptr(t):
    if t is None:
        return None
    if isinstance(t, int):
        return t
    return t.data_ptr()


def _stream(s):
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return s.cuda_stream


class Heap:
    """One batched min-heap on the current CUDA device.

    Heap(batch_num, batch_size, init_limits) as in the reference
    (heap/tditdd/heap.cuh:33-67): batch_num full nodes of batch_size sorted
    keys plus the partial buffer (node 0).  Every key must be strictly below
    init_limits (default: the key type's maximum).
    """

    def __init__(self, batch_num, batch_size, init_limits=None, *, key="u32", variant="bottomup",
                 partial_buffer=True):
        if key not in KEY_KINDS:
            raise ValueError(f"key must be one of {sorted(KEY_KINDS)}")
        if variant not in _VARIANTS:
            raise ValueError(f"variant must be one of {sorted(_VARIANTS)}")
        self.key = key
        self.variant = "topdown" if _VARIANTS[variant] == 0 else "bottomup"
        self.partial_buffer = bool(partial_buffer)
        self.batch_num = int(batch_num)
        self.batch_size = int(batch_size)
        self.key_bytes = _KEY_BYTES[key]
        self._h = _VP()
        lim = None
        if init_limits is not None:
            lim = _KEY_CTYPE[key](init_limits)
        _check(lib().gh_heap_create(ctypes.byref(self._h), KEY_KINDS[key], _VARIANTS[variant],
                                    1 if partial_buffer else 0, self.batch_num, self.batch_size,
                                    ctypes.byref(lim) if lim is not None else None), "Heap()")
        if init_limits is None:
            init_limits = {"u32": 2**32 - 1, "i32": 2**31 - 1, "u64": 2**64 - 1}[key]
        self.init_limits = int(init_limits)

    # ---------------------------------------------------------------- lifetime
    def close(self):
        if self._h:
            lib().gh_heap_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def reset(self, stream=None):
        """reset(): heap/tditdd/heap.cuh:69-91."""
        _check(lib().gh_heap_reset(self._h, _stream(stream)), "reset")
        _check(lib().gh_heap_sync(self._h, _stream(stream)), "reset")

    def reset_async(self, stream=None):
        """reset() queued on `stream` without waiting."""
        _check(lib().gh_heap_reset(self._h, _stream(stream)), "reset")

    # ---------------------------------------------------------------- tuning
    def set_timeout(self, seconds):
        _check(lib().gh_heap_set_timeout(self._h, float(seconds)), "set_timeout")

    def set_block_threads(self, threads):
        _check(lib().gh_heap_set_block_threads(self._h, int(threads)), "set_block_threads")

    def set_grid(self, blocks):
        _check(lib().gh_heap_set_grid(self._h, int(blocks)), "set_grid")

    def info(self):
        vals = [_I() for _ in range(7)]
        _check(lib().gh_heap_info(self._h, *[ctypes.byref(v) for v in vals]), "info")
        names = ["key_kind", "variant", "partial_buffer", "batch_num", "batch_size", "block_threads", "grid"]
        return {n: v.value for n, v in zip(names, vals)}

    # ---------------------------------------------------------------- operations
    def insertion(self, items, size, stream=None):
        """One Heap::insertion(items, size) by one block (heap/tditdd/heap.cuh:536)."""
        _check(lib().gh_heap_insert_batch(self._h, _ptr(items), int(size), _stream(stream)), "insertion")

    def delete_root(self, items, stream=None):
        """One deleteRoot (+ deleteUpdate) by one block; HEAP_SORT output at
        items + the heap's output cursor.  Returns the number of keys written."""
        sz = _I()
        _check(lib().gh_heap_delete_batch(self._h, _ptr(items), ctypes.byref(sz), _stream(stream)), "deleteRoot")
        return sz.value

    def retrieve(self, out, size, stream=None):
        """retrieve(ret, *size) by one block (applications/sssp_longfei_new/
        heap.cuh:79-270): the `size` smallest keys (at most one batch) into
        out[0, n), ascending; returns n.  Heaps with the partial buffer."""
        got = _I()
        _check(lib().gh_heap_retrieve(self._h, _ptr(out), int(size), ctypes.byref(got), _stream(stream)),
               "retrieve")
        return got.value

    def insert(self, keys, n=None, chunk=0, stream=None):
        """Bulk insertion of n keys in insertion() calls of `chunk` keys over
        the heap's grid (insertKernel, test/heap_test.cu:44-58).  Asynchronous."""
        n = keys.numel() if n is None else int(n)
        _check(lib().gh_heap_insert(self._h, _ptr(keys), n, int(chunk), _stream(stream)), "insert")

    def delete(self, out, max_keys=None, stream=None, sync=True):
        """Deletes until empty (deleteKernel, test/heap_test.cu:60-77) into
        out[0, n) in ascending order; returns n (None when sync=False)."""
        max_keys = out.numel() if max_keys is None else int(max_keys)
        if not sync:
            _check(lib().gh_heap_delete(self._h, _ptr(out), max_keys, None, _stream(stream)), "delete")
            return None
        got = _LL()
        _check(lib().gh_heap_delete(self._h, _ptr(out), max_keys, ctypes.byref(got), _stream(stream)), "delete")
        return got.value

    def delete_below(self, out, threshold, max_keys=None, stream=None):
        """deleteRoot(items, size, app_t_val) until the smallest key is not
        below `threshold` (artifacts/astar/BGPQ_B/heap.cuh:260-289): whole
        batches into out[0, n) in ascending order; returns n."""
        max_keys = out.numel() if max_keys is None else int(max_keys)
        t = _KEY_CTYPE[self.key](threshold)
        got = _LL()
        _check(lib().gh_heap_delete_below(self._h, _ptr(out), max_keys, ctypes.byref(t), ctypes.byref(got),
                                          _stream(stream)), "delete_below")
        return got.value

    def gc(self, threshold=None, stream=None):
        """Garbage collection (invalidFilter, artifacts/astar/gc.cuh:77-180):
        keeps the keys below `threshold` (None: every real key) and rebuilds
        the heap from them on the device; returns the number kept."""
        t = _KEY_CTYPE[self.key](threshold) if threshold is not None else None
        kept = _LL()
        _check(lib().gh_heap_gc(self._h, ctypes.byref(t) if t is not None else None, ctypes.byref(kept),
                                _stream(stream)), "gc")
        return kept.value

    def concurrent(self, keys, out, n=None, chunk=0, max_keys=None, stream=None):
        """concurrentKernel (test/heap_test.cu:13-38): half the grid inserts
        keys[0, n) while the other half makes n // batch_size deletes into
        out; returns the number of keys deleted."""
        n = keys.numel() if n is None else int(n)
        max_keys = out.numel() if max_keys is None else int(max_keys)
        got = _LL()
        _check(lib().gh_heap_concurrent(self._h, _ptr(keys), n, int(chunk), _ptr(out), max_keys, ctypes.byref(got),
                                        _stream(stream)), "concurrent")
        return got.value

    def sort(self, keys, out, n=None, stream=None):
        """Heap-sort: reset, insert all keys, delete all (test/partial_heap_test.cu:88-176)."""
        n = keys.numel() if n is None else int(n)
        _check(lib().gh_heap_sort(self._h, _ptr(keys), n, _ptr(out), _stream(stream)), "sort")

    def sort_host(self, keys, out, n=None, stream=None):
        """Heap-sort with host buffers (gh_heap_sort_host): keys and out are
        CPU tensors (pinned for overlap) or numpy arrays; the copies overlap
        the inserts and deletes.  Queued on `stream`; sync() waits."""
        if hasattr(keys, "data_ptr"):
            kp, op = keys.data_ptr(), out.data_ptr()
            n = keys.numel() if n is None else int(n)
        else:
            kp, op = keys.ctypes.data, out.ctypes.data
            n = keys.size if n is None else int(n)
        _check(lib().gh_heap_sort_host(self._h, kp, n, op, _stream(stream)), "sort_host")

    def sync(self, stream=None):
        _check(lib().gh_heap_sync(self._h, _stream(stream)), "sync")

    # ---------------------------------------------------------------- inspection
    def check_insert_heap(self, stream=None):
        """checkInsertHeap() on the device; returns (ok, message)."""
        ok = _I()
        msg = ctypes.create_string_buffer(256)
        _check(lib().gh_heap_check(self._h, ctypes.byref(ok), msg, 256, _stream(stream)), "checkInsertHeap")
        return bool(ok.value), msg.value.decode()

    def checkInsertHeap(self):
        return self.check_insert_heap()[0]

    def item_count(self):
        n = _LL()
        _check(lib().gh_heap_item_count(self._h, ctypes.byref(n)), "itemCount")
        return n.value

    def node_count(self):
        n = _I()
        _check(lib().gh_heap_node_count(self._h, ctypes.byref(n)), "nodeCount")
        return n.value

    def is_empty(self):
        e = _I()
        _check(lib().gh_heap_is_empty(self._h, ctypes.byref(e)), "isEmpty")
        return bool(e.value)

    itemCount = item_count
    nodeCount = node_count
    isEmpty = is_empty

    def snapshot(self):
        """(items, status, counters) as numpy arrays; counters =
        [batchCount, partialBufferSize, deleteCount, err, errOp, errNode, errState]."""
        import numpy as np
        dt = {"u32": np.uint32, "i32": np.int32, "u64": np.uint64}[self.key]
        items = np.empty((self.batch_num + 1) * self.batch_size, dt)
        status = np.empty(self.batch_num + 1, np.int32)
        counters = np.zeros(7, np.int32)
        _check(lib().gh_heap_snapshot(self._h, items.ctypes.data, status.ctypes.data, counters.ctypes.data),
               "snapshot")
        return items, status, counters

    def restore(self, items, counters):
        """Puts back a snapshot's items and counters (from this heap or one of
        the same shape) with every lock free and the error record cleared."""
        import numpy as np
        dt = {"u32": np.uint32, "i32": np.int32, "u64": np.uint64}[self.key]
        items = np.ascontiguousarray(items, dt)
        if items.size != (self.batch_num + 1) * self.batch_size:
            raise ValueError(f"restore: {items.size} keys for a heap of {(self.batch_num + 1) * self.batch_size}")
        c = np.ascontiguousarray(np.asarray(counters, np.int32)[:3])
        _check(lib().gh_heap_restore(self._h, items.ctypes.data, c.ctypes.data), "restore")

    OWNER_STATS = ("deletes", "wait_carried", "wait_lent", "wait_ring", "plan", "pass", "general_steps", "loop",
                   "take_lock", "take_load", "take_idle", "lends", "reloads", "plan_read", "pass_work", "pass_sync")

    def set_owner_depth(self, depth):
        """Owner-mode bulk delete depth: -1 automatic, 0 off, 2..4 resident levels."""
        _check(lib().gh_heap_set_owner_depth(self._h, int(depth)), "set_owner_depth")

    def owner_stats(self):
        """Counters of the last owner-mode bulk delete (SM cycles unless a count)."""
        import numpy as np
        buf = np.zeros(len(self.OWNER_STATS), np.uint64)
        _check(lib().gh_heap_owner_stats(self._h, buf.ctypes.data, buf.size), "owner_stats")
        return dict(zip(self.OWNER_STATS, (int(v) for v in buf)))

    def inject_lock(self, node, state):
        """Fault injection: leave node's lock word in `state` (tests of the bounded waits)."""
        _check(lib().gh_heap_inject_lock(self._h, int(node), int(state)), "inject_lock")

    def device_view(self):
        """Bytes of the gh::Heap<K, variant, partial_buffer> device view."""
        n = lib().gh_heap_view_bytes()
        buf = ctypes.create_string_buffer(n)
        _check(lib().gh_heap_device_view(self._h, buf, n), "device_view")
        return buf.raw

    @staticmethod
    def smem_bytes(key, batch_size):
        return lib().gh_heap_smem_bytes(KEY_KINDS[key], int(batch_size))
