"""ctypes access to the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU leg of bench.py, as the checker -- never by the product path.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

DISTS = {"uniform": 0, "sorted": 1, "reverse": 2, "zipf": 3}
DTYPES = {"u32": np.uint32, "u64": np.uint64, "i32": np.int32}
CTYPES = {"u32": ctypes.c_uint32, "u64": ctypes.c_uint64, "i32": ctypes.c_int32}
INIT = {"u32": 2**32 - 1, "u64": 2**64 - 1, "i32": 2**31 - 1}
_VP = ctypes.c_void_p
_lib = None


def lib():
    global _lib
    if _lib is None:
        src = [os.path.join(HERE, f) for f in ("bgpq_oracle.cpp", "search_oracle.cpp", "bgpq_oracle.h")]
        if not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
            subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
        so = ctypes.CDLL(LIB)
        for k in DTYPES:
            getattr(so, f"gho_gen_{k}").argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64, _VP, ctypes.c_int]
            getattr(so, f"gho_sort_{k}").argtypes = [_VP, ctypes.c_uint64, ctypes.c_int]
            getattr(so, f"gho_check_{k}").argtypes = [ctypes.c_int, _VP, _VP, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
            f = getattr(so, f"gho_model_create_{k}")
            f.restype = _VP
            f.argtypes = [ctypes.c_int] * 4 + [CTYPES[k]]
            getattr(so, f"gho_model_insert_{k}").argtypes = [_VP, _VP, ctypes.c_int]
            getattr(so, f"gho_model_delete_{k}").argtypes = [_VP, _VP]
            getattr(so, f"gho_model_state_{k}").argtypes = [_VP, _VP, _VP]
        so.gho_model_destroy.argtypes = [_VP]
        so.gho_reversed_idx.restype = ctypes.c_uint32
        so.gho_reversed_idx.argtypes = [ctypes.c_uint32]
        so.gho_dijkstra.argtypes = [ctypes.c_int, _VP, _VP, _VP, ctypes.c_int, _VP]
        so.gho_dijkstra_many.argtypes = [ctypes.c_int, _VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int, _VP]
        so.gho_astar_grid.restype = ctypes.c_uint32
        so.gho_astar_grid.argtypes = [ctypes.c_int, ctypes.c_int, _VP, _VP, _VP]
        so.gho_astar_grid8_sg.restype = ctypes.c_uint32
        so.gho_astar_grid8_sg.argtypes = [ctypes.c_int, ctypes.c_int, _VP, ctypes.c_int, ctypes.c_int, _VP]
        so.gho_astar_grid8.restype = ctypes.c_uint32
        so.gho_astar_grid8.argtypes = [ctypes.c_int, ctypes.c_int, _VP, _VP]
        so.gho_astar_ref8.restype = ctypes.c_uint32
        so.gho_astar_ref8.argtypes = [ctypes.c_int, ctypes.c_int, _VP]
        so.gho_astar_grid_sg.restype = ctypes.c_uint32
        so.gho_astar_grid_sg.argtypes = [ctypes.c_int, ctypes.c_int, _VP, ctypes.c_int, ctypes.c_int, _VP, _VP]
        so.gho_astar_grid_many.argtypes = [ctypes.c_int, _VP, _VP, _VP, _VP, ctypes.c_int, _VP]
        so.gho_knap_bb.restype = ctypes.c_longlong
        so.gho_knap_bb.argtypes = [ctypes.c_int, _VP, _VP, ctypes.c_longlong, _VP, _VP]
        so.gho_knap_dp.restype = ctypes.c_longlong
        so.gho_knap_dp.argtypes = [ctypes.c_int, _VP, _VP, ctypes.c_longlong]
        so.gho_knap_bb_many.argtypes = [ctypes.c_int, _VP, _VP, _VP, _VP, _VP, ctypes.c_int, _VP]
        so.gho_sort_bytes.restype = ctypes.c_double
        so.gho_sort_bytes.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _lib = so
    return _lib


def gen(key, seed, dist, n, threads=None):
    """Seeded keys of the plain heap-sort workload (see bgpq_oracle.h)."""
    out = np.empty(n, DTYPES[key])
    th = threads or os.cpu_count() or 1
    getattr(lib(), f"gho_gen_{key}")(seed, DISTS[dist], n, out.ctypes.data, th)
    return out


def sort(a, threads=1):
    """std::sort (threads > 1: per-thread std::sort + pairwise std::merge), in place."""
    key = {np.dtype(np.uint32): "u32", np.dtype(np.uint64): "u64", np.dtype(np.int32): "i32"}[a.dtype]
    assert a.flags.c_contiguous
    getattr(lib(), f"gho_sort_{key}")(a.ctypes.data, a.size, threads)
    return a


def check_heap(variant, items, status, batch_size, batch_count, partial_size):
    """checkInsertHeap restated; returns (ok, message)."""
    key = {np.dtype(np.uint32): "u32", np.dtype(np.uint64): "u64", np.dtype(np.int32): "i32"}[items.dtype]
    msg = ctypes.create_string_buffer(200)
    v = 0 if variant in ("topdown", "td", 0) else 1
    st = None if status is None else np.ascontiguousarray(status, np.int32)
    ok = getattr(lib(), f"gho_check_{key}")(v, items.ctypes.data, None if st is None else st.ctypes.data,
                                            int(batch_size), int(batch_count), int(partial_size), msg, 200)
    return Result(bool(ok), msg.value.decode())


class Result(tuple):
    def __new__(cls, ok, msg):
        return tuple.__new__(cls, (ok, msg))

    def __bool__(self):
        return self[0]


def reversed_idx(i):
    return lib().gho_reversed_idx(i)


def dijkstra(rowptr, col, w, sources, threads=1):
    """CPU Dijkstra (std::priority_queue on dist<<32|v) from each source;
    returns a (len(sources), n) uint32 array, UINT32_MAX = unreachable."""
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    w = np.ascontiguousarray(w, np.uint32)
    src = np.ascontiguousarray(np.atleast_1d(sources), np.int32)
    n = rowptr.size - 1
    out = np.empty((src.size, n), np.uint32)
    lib().gho_dijkstra_many(n, rowptr.ctypes.data, col.ctypes.data, w.ctypes.data, src.ctypes.data, src.size,
                            threads, out.ctypes.data)
    return out


def astar_ref8(bitmap_words, width, height):
    """The reference's 8-connected bitmap A* restated (gho_astar_ref8):
    bitmap_words is a uint32 array, bit i set = cell i open."""
    import numpy as np
    words = np.ascontiguousarray(bitmap_words, np.uint32)
    return int(lib().gho_astar_ref8(int(width), int(height), words.ctypes.data))


def astar_grid8(open_cells):
    """Optimal cost from (0, 0) to the last cell on the reference's map
    model (gho_astar_grid8): open_cells (h, w) nonzero = open, eight moves
    costing 3 2 2 2 1 3 1 2; UINT32_MAX if unreachable."""
    import numpy as np
    g = np.ascontiguousarray(open_cells, np.uint8)
    return int(lib().gho_astar_grid8(g.shape[1], g.shape[0], g.ctypes.data, None))


def astar_grid8_sg(open_cells, start, goal):
    """As astar_grid8, from cell `start` to cell `goal` (Manhattan heuristic to the goal)."""
    import numpy as np
    g = np.ascontiguousarray(open_cells, np.uint8)
    return int(lib().gho_astar_grid8_sg(g.shape[1], g.shape[0], g.ctypes.data, int(start), int(goal), None))


def astar_grid(cost, stats=False):
    """Optimal 4-connected path cost over a (height, width) uint8 cost grid
    (0 = obstacle) from the top-left to the bottom-right cell; UINT32_MAX when
    unreachable.  stats=True also returns (expansions, max_open)."""
    cost = np.ascontiguousarray(cost, np.uint8)
    h, w = cost.shape
    e, m = ctypes.c_longlong(), ctypes.c_longlong()
    r = lib().gho_astar_grid(w, h, cost.ctypes.data, ctypes.byref(e), ctypes.byref(m))
    return (r, e.value, m.value) if stats else r


def astar_grid_sg(cost, start, goal):
    """Optimal path cost between cells start and goal (y * width + x)."""
    cost = np.ascontiguousarray(cost, np.uint8)
    h, w = cost.shape
    return lib().gho_astar_grid_sg(w, h, cost.ctypes.data, int(start), int(goal), None, None)


def astar_grid_many(grids, threads=None):
    """Optimal costs of a list of (height, width) uint8 grids, one per task."""
    th = threads or os.cpu_count() or 1
    widths = np.asarray([g.shape[1] for g in grids], np.int32)
    heights = np.asarray([g.shape[0] for g in grids], np.int32)
    offsets = np.zeros(len(grids), np.int64)
    offsets[1:] = np.cumsum([g.size for g in grids])[:-1]
    flat = np.ascontiguousarray(np.concatenate([g.ravel() for g in grids])) if grids else np.zeros(1, np.uint8)
    out = np.zeros(len(grids), np.uint32)
    lib().gho_astar_grid_many(len(grids), widths.ctypes.data, heights.ctypes.data, offsets.ctypes.data,
                              flat.ctypes.data, th, out.ctypes.data)
    return out


def knap_bb(w, p, cap, stats=False):
    """0/1 knapsack optimum by best-first branch-and-bound (Dantzig bound)."""
    w = np.ascontiguousarray(w, np.int32)
    p = np.ascontiguousarray(p, np.int32)
    nodes, mo = ctypes.c_longlong(), ctypes.c_longlong()
    r = lib().gho_knap_bb(w.size, w.ctypes.data, p.ctypes.data, int(cap), ctypes.byref(nodes), ctypes.byref(mo))
    return (r, nodes.value, mo.value) if stats else r


def knap_dp(w, p, cap):
    """0/1 knapsack optimum by the capacity dynamic program."""
    w = np.ascontiguousarray(w, np.int32)
    p = np.ascontiguousarray(p, np.int32)
    return lib().gho_knap_dp(w.size, w.ctypes.data, p.ctypes.data, int(cap))


def knap_bb_many(instances, threads=None):
    """Optima of a list of (w, p, cap) instances, one per task."""
    th = threads or os.cpu_count() or 1
    sizes = np.asarray([len(w) for w, _, _ in instances], np.int32)
    offsets = np.zeros(len(instances), np.int64)
    offsets[1:] = np.cumsum(sizes)[:-1]
    W = np.ascontiguousarray(np.concatenate([w for w, _, _ in instances]), np.int32)
    P = np.ascontiguousarray(np.concatenate([p for _, p, _ in instances]), np.int32)
    caps = np.asarray([c for _, _, c in instances], np.int64)
    out = np.zeros(len(instances), np.int64)
    lib().gho_knap_bb_many(len(instances), sizes.ctypes.data, offsets.ctypes.data, W.ctypes.data, P.ctypes.data,
                           caps.ctypes.data, th, out.ctypes.data)
    return out


def sort_bytes(n, batch_size, key_bytes, partial_buffer):
    """Algorithmic node traffic of one heap-sort in bytes."""
    return lib().gho_sort_bytes(n, batch_size, key_bytes, 1 if partial_buffer else 0)


class Model:
    """Sequential Heap<K> model (insertion / deleteRoot+deleteUpdate)."""

    def __init__(self, key, variant, partial_buffer, batch_num, batch_size, init_limits=None):
        self.key = key
        self.dt = DTYPES[key]
        self.batch_num = batch_num
        self.batch_size = batch_size
        v = 0 if variant in ("topdown", "td", 0) else 1
        lim = INIT[key] if init_limits is None else init_limits
        self.h = getattr(lib(), f"gho_model_create_{key}")(v, 1 if partial_buffer else 0, batch_num, batch_size,
                                                          CTYPES[key](lim))

    def insert(self, items):
        items = np.ascontiguousarray(items, self.dt)
        return getattr(lib(), f"gho_model_insert_{self.key}")(self.h, items.ctypes.data, items.size)

    def delete(self, out):
        assert out.dtype == self.dt and out.flags.c_contiguous
        return getattr(lib(), f"gho_model_delete_{self.key}")(self.h, out.ctypes.data)

    def state(self):
        items = np.empty((self.batch_num + 1) * self.batch_size, self.dt)
        counters = np.zeros(3, np.int32)
        getattr(lib(), f"gho_model_state_{self.key}")(self.h, items.ctypes.data, counters.ctypes.data)
        return items, counters

    def __del__(self):
        try:
            lib().gho_model_destroy(self.h)
        except Exception:
            pass


class FifoModel:
    """Sequential restatement of the reference's Buffer<K>
    (artifacts/buffer/buffer.cuh:6-218) for replaying single-block runs.

    Positions begin <= read <= write <= end count keys since creation; a slot
    is position % capacity.  insertToBuffer (buffer.cuh:127-170) reserves
    [end, end + size), needs end + size - begin <= capacity, writes the keys
    and publishes by moving write to its end.  deleteFromBuffer
    (buffer.cuh:172-214) claims min(max, write - read) keys at read, copies
    them out and frees them by moving begin.  With one block every wait
    succeeds at once, so this model is exact for it.
    """

    def __init__(self, capacity, dtype=np.uint32):
        cap = 1
        while cap < capacity:
            cap <<= 1
        self.capacity = cap
        self.ring = np.zeros(cap, dtype)
        self.begin = self.read = self.write = self.end = 0

    def insert(self, keys):
        size = len(keys)
        if size == 0:
            return
        start = self.end
        if start + size - self.begin > self.capacity:
            raise OverflowError("ring full: a lone pusher would wait forever")
        self.end += size
        idx = (start + np.arange(size)) % self.capacity
        self.ring[idx] = keys
        assert self.write == start
        self.write = start + size

    def delete(self, max_size):
        n = min(max_size, self.write - self.read)
        start = self.read
        self.read += n
        out = self.ring[(start + np.arange(n)) % self.capacity].copy()
        assert self.begin == start
        self.begin = start + n
        return out

    def push(self, keys, chunk):
        """insertKernel with one block: pieces of `chunk` keys in order."""
        for off in range(0, len(keys), chunk):
            self.insert(keys[off:off + chunk])

    def pop(self, max_keys, chunk):
        """deleteKernel with one block: takes until max_keys or empty."""
        parts = []
        taken = 0
        while taken < max_keys:
            got = self.delete(min(chunk, max_keys - taken))
            if len(got) == 0:
                break
            parts.append(got)
            taken += len(got)
        return np.concatenate(parts) if parts else self.ring[:0].copy()

    def positions(self):
        return (self.begin, self.read, self.write, self.end)


def fifo_pieces_ok(inp, out, piece_starts):
    """Checks a multi-block FIFO run: `out` is a permutation of `inp` (distinct
    keys) in which every piece [piece_starts[i], piece_starts[i+1]) of the
    input appears whole and in order (a piece is one insertToBuffer call)."""
    inp = np.asarray(inp)
    out = np.asarray(out)
    if len(inp) != len(out) or not np.array_equal(np.sort(inp), np.sort(out)):
        return False
    pos = np.empty(len(out), np.int64)
    order = np.argsort(out, kind="stable")
    rank_in = np.argsort(np.argsort(inp, kind="stable"), kind="stable")
    pos[:] = order[rank_in]  # pos[i] = index in out of inp[i]
    cont = np.ones(len(inp), bool)
    cont[np.asarray(piece_starts, np.int64)[np.asarray(piece_starts) < len(inp)]] = False
    return bool(np.all(pos[1:][cont[1:]] == pos[:-1][cont[1:]] + 1))


def fifo_piece_starts(n, chunk, split):
    """Input indices where insertToBuffer calls start for n keys pushed in
    pieces of `chunk` (split: each piece as its first third and the rest,
    bufferTest.cu:19-24)."""
    starts = []
    for off in range(0, n, chunk):
        size = min(chunk, n - off)
        starts.append(off)
        if split and size // 3 > 0:
            starts.append(off + size // 3)
    return np.asarray(starts, np.int64)
