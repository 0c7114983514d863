"""Device FIFO buffer over the C ABI (include/gpuheap_fifo.h).

Host-side mirror of the reference's Buffer<K> (artifacts/buffer/buffer.cuh:
6-218) and its test driver's kernels (artifacts/buffer/bufferTest.cu:13-56):
a ring of `capacity` keys (rounded up to a power of two) with the positions
begin <= read <= write <= end.  Device buffers are torch CUDA tensors (or raw
device pointers); there is no CPU fallback.
"""
import ctypes

from . import KEY_KINDS, _I, _LL, _VP, _check, _ptr, _stream, lib

__all__ = ["Fifo"]


class Fifo:
    """Buffer<K>(capacity) on the current CUDA device."""

    def __init__(self, capacity, key="u32"):
        if key not in KEY_KINDS:
            raise ValueError(f"key must be one of {sorted(KEY_KINDS)}")
        self.key = key
        self._f = _VP()
        _check(lib().gh_fifo_create(ctypes.byref(self._f), KEY_KINDS[key], int(capacity)), "Buffer()")
        self.capacity = self.info()["capacity"]

    def close(self):
        if self._f:
            lib().gh_fifo_destroy(self._f)
            self._f = _VP()

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
        _check(lib().gh_fifo_reset(self._f, _stream(stream)), "reset")

    def set_timeout(self, seconds):
        _check(lib().gh_fifo_set_timeout(self._f, float(seconds)), "set_timeout")

    def set_launch(self, blocks=0, threads=0):
        _check(lib().gh_fifo_set_launch(self._f, int(blocks), int(threads)), "set_launch")

    def push(self, keys, n=None, chunk=0, stream=None):
        """insertKernel (bufferTest.cu:39-47): appends keys[0, n) in pieces of
        `chunk` keys, one insertToBuffer per piece.  Asynchronous."""
        n = keys.numel() if n is None else int(n)
        _check(lib().gh_fifo_push(self._f, _ptr(keys), n, int(chunk), _stream(stream)), "insertToBuffer")

    def pop(self, out, max_keys=None, chunk=0, stream=None, sync=True):
        """deleteKernel (bufferTest.cu:49-56): takes up to max_keys keys in
        FIFO order into out[0, n); returns n (None when sync=False)."""
        max_keys = out.numel() if max_keys is None else int(max_keys)
        if not sync:
            _check(lib().gh_fifo_pop(self._f, _ptr(out), max_keys, int(chunk), None, _stream(stream)),
                   "deleteFromBuffer")
            return None
        got = _LL()
        _check(lib().gh_fifo_pop(self._f, _ptr(out), max_keys, int(chunk), ctypes.byref(got), _stream(stream)),
               "deleteFromBuffer")
        return got.value

    def concurrent(self, keys, out, n=None, chunk=0, max_keys=None, stream=None):
        """concurrentKernel (bufferTest.cu:13-37): half the blocks push
        keys[0, n) while the other half take max_keys keys into out."""
        n = keys.numel() if n is None else int(n)
        max_keys = out.numel() if max_keys is None else int(max_keys)
        got = _LL()
        _check(lib().gh_fifo_concurrent(self._f, _ptr(keys), n, int(chunk), _ptr(out), max_keys, ctypes.byref(got),
                                        _stream(stream)), "concurrent")
        return got.value

    def count(self):
        n = _LL()
        _check(lib().gh_fifo_count(self._f, ctypes.byref(n)), "count")
        return n.value

    def positions(self):
        """printBufferPtr (buffer.cuh:88-96): (begin, read, write, end)."""
        v = [ctypes.c_ulonglong() for _ in range(4)]
        _check(lib().gh_fifo_positions(self._f, *[ctypes.byref(x) for x in v]), "positions")
        return tuple(x.value for x in v)

    def snapshot(self):
        """printBuffer (buffer.cuh:98-123): (ring items, positions) as numpy."""
        import numpy as np
        dt = {"u32": np.uint32, "i32": np.int32, "u64": np.uint64}[self.key]
        items = np.empty(self.capacity, dt)
        pos = np.zeros(4, np.uint64)
        _check(lib().gh_fifo_snapshot(self._f, items.ctypes.data, pos.ctypes.data), "snapshot")
        return items, pos

    def inject_reservation(self, n):
        """Failure injection: a reservation of n slots that is never published."""
        _check(lib().gh_fifo_inject_reservation(self._f, int(n)), "inject_reservation")

    def device_view(self):
        n = lib().gh_fifo_view_bytes()
        buf = ctypes.create_string_buffer(n)
        _check(lib().gh_fifo_device_view(self._f, buf, n), "device_view")
        return buf.raw

    def info(self):
        kind, cap, blocks, threads, site = _I(), _LL(), _I(), _I(), _I()
        _check(lib().gh_fifo_info(self._f, ctypes.byref(kind), ctypes.byref(cap), ctypes.byref(blocks),
                                  ctypes.byref(threads), ctypes.byref(site)), "info")
        return {"key_kind": kind.value, "capacity": cap.value, "blocks": blocks.value, "threads": threads.value,
                "err_site": site.value}
