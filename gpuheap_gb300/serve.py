"""Served SSSP and grid A* queries: a continuous-batching loop (gh_serve_*).

Server wraps the C ABI: resident graphs and maps, submit(), step(),
result().  run_stream() drives it with a Poisson arrival process: on every
turn it submits the queries whose arrival time has passed, runs one step
(admission by free memory, one launch over every admitted query, collection
of the finished ones) and stamps the finished queries; latency is finish
time minus arrival time.  run_plain() is the baseline: the same queries one
at a time, each run alone to its end before the next is submitted.
"""
import ctypes
import time

import numpy as np

from . import _check, _I, _LL, _VP, lib

SSSP, ASTAR = 2, 0
_VARIANTS = {"topdown": 0, "bottomup": 1}
QUEUED, ADMITTED, FINISHED, FAILED = 0, 1, 2, 3


class Server:
    def __init__(self, arena_bytes=0, max_slots=256, batch_size=512, variant="bottomup", batches_per_step=8,
                 sssp_vertices_per_block=1 << 15, sssp_max_blocks=24, astar_cells_per_block=1 << 18,
                 astar_max_blocks=8):
        h = _VP()
        _check(lib().gh_serve_create(ctypes.byref(h), int(arena_bytes), max_slots, batch_size, _VARIANTS[variant],
                                     batches_per_step), "serve_create")
        self._h = h
        self._keep = []  # the datasets' device arrays must outlive the server
        try:
            _check(lib().gh_serve_set_blocks(h, int(sssp_vertices_per_block), int(sssp_max_blocks),
                                             int(astar_cells_per_block), int(astar_max_blocks)), "serve_set_blocks")
        except Exception:
            self.close()
            raise

    def add_graph(self, graph):
        """A resident CSR graph (gpuheap_gb300.sssp.Graph); returns its id."""
        i = _I()
        _check(lib().gh_serve_add_graph(self._h, graph.n, graph.rowptr.data_ptr(), graph.col.data_ptr(),
                                        graph.w.data_ptr(), ctypes.byref(i)), "serve_add_graph")
        self._keep.append(graph)
        return i.value

    def add_map(self, cost):
        """A resident (height, width) uint8 cost grid (torch tensor on the device); returns its id."""
        i = _I()
        h, w = cost.shape
        _check(lib().gh_serve_add_map(self._h, w, h, cost.data_ptr(), ctypes.byref(i)), "serve_add_map")
        self._keep.append(cost)
        return i.value

    def add_bitmap(self, open_cells):
        """A resident (height, width) uint8 map on the reference's model
        (nonzero = open, eight moves with its direction costs); returns its id."""
        i = _I()
        h, w = open_cells.shape
        _check(lib().gh_serve_add_bitmap(self._h, w, h, open_cells.data_ptr(), ctypes.byref(i)), "serve_add_bitmap")
        self._keep.append(open_cells)
        return i.value

    def submit(self, kind, dataset, a, b=0):
        """Queues SSSP (kind SSSP, from vertex a) or A* (kind ASTAR, cell a to cell b); returns the query id."""
        q = _LL()
        _check(lib().gh_serve_submit(self._h, kind, dataset, int(a), int(b), ctypes.byref(q)), "serve_submit")
        return q.value

    def step(self, stream=None):
        """One step; returns (ids finished in it, active, queued)."""
        f, a, qd = _I(), _I(), _I()
        _check(lib().gh_serve_step(self._h, _stream(stream), ctypes.byref(f), ctypes.byref(a), ctypes.byref(qd)),
               "serve_step")
        ids = (_LL * max(1, f.value))()
        n = _I()
        _check(lib().gh_serve_finished(self._h, ids, f.value, ctypes.byref(n)), "serve_finished")
        return [ids[i] for i in range(f.value)], a.value, qd.value

    def start(self, idle_ms=100):
        """Switches to the device-resident loop: from now on submit() posts
        into a pinned request ring and poll() collects completions; the
        loop's launch leaves after idle_ms without work and poll() launches
        it again when work arrives."""
        _check(lib().gh_serve_start(self._h, int(idle_ms)), "serve_start")

    def poll(self):
        """Device loop: completions since the last poll; returns (ids
        finished, active, queued).  Does not block."""
        f, a, qd = _I(), _I(), _I()
        _check(lib().gh_serve_poll(self._h, ctypes.byref(f), ctypes.byref(a), ctypes.byref(qd)), "serve_poll")
        ids = (_LL * max(1, f.value))()
        n = _I()
        _check(lib().gh_serve_finished(self._h, ids, f.value, ctypes.byref(n)), "serve_finished")
        return [ids[i] for i in range(f.value)], a.value, qd.value

    def stop(self):
        """Device loop: pauses it (the launch leaves after its blocks'
        current stints); start() resumes the queries left in it."""
        _check(lib().gh_serve_stop(self._h), "serve_stop")

    def result(self, q):
        """(state, r0, r1, finish step): SSSP r0 = reachable vertices, r1 = sum
        of their distances; A* r0 = optimal cost (UINT32_MAX unreachable)."""
        st, r0, r1, fs = _I(), ctypes.c_ulonglong(), ctypes.c_ulonglong(), _LL()
        _check(lib().gh_serve_result(self._h, int(q), ctypes.byref(st), ctypes.byref(r0), ctypes.byref(r1),
                                     ctypes.byref(fs)), "serve_result")
        return st.value, r0.value, r1.value, fs.value

    def info(self):
        u, f, s, n = _LL(), _LL(), _I(), _LL()
        _check(lib().gh_serve_info(self._h, ctypes.byref(u), ctypes.byref(f), ctypes.byref(s), ctypes.byref(n)),
               "serve_info")
        return {"used_bytes": u.value, "free_bytes": f.value, "slots_used": s.value, "steps": n.value}

    def close(self):
        if getattr(self, "_h", None):
            lib().gh_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream(s):
    if s is None:
        return None
    return s.cuda_stream if hasattr(s, "cuda_stream") else s


def poisson_arrivals(count, rate, seed):
    """Arrival times (s) of `count` requests at `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, count))


def run_stream(server, queries, arrivals, stream=None, max_seconds=600.0, resident=False):
    """Serves `queries` ((kind, dataset, a, b) tuples) arriving at `arrivals`
    (seconds from the start), through host steps or, with resident=True,
    through the device loop (the server must have been started).  Returns
    (latency seconds per query, results per query, makespan seconds, steps
    or polls)."""
    n = len(queries)
    ids = [None] * n
    finish = np.full(n, np.nan)
    byid = {}
    t0 = time.perf_counter()
    nxt = done = steps = 0
    while done < n:
        now = time.perf_counter() - t0
        if now > max_seconds:
            raise RuntimeError(f"served stream did not finish in {max_seconds} s")
        while nxt < n and arrivals[nxt] <= now:
            k, d, a, b = queries[nxt]
            ids[nxt] = server.submit(k, d, a, b)
            byid[ids[nxt]] = nxt
            nxt += 1
        if done == nxt:  # nothing in the system: wait for the next arrival
            time.sleep(max(0.0, min(arrivals[nxt] - now, 0.001)))
            continue
        fin, _, _ = server.poll() if resident else server.step(stream)
        steps += 1
        t = time.perf_counter() - t0
        for q in fin:
            finish[byid[q]] = t
            done += 1
    makespan = time.perf_counter() - t0
    results = [server.result(q) for q in ids]
    return finish - np.asarray(arrivals[:n]), results, makespan, steps


def run_plain(server, queries, stream=None):
    """Each query alone: submit it, step until it finishes.  Returns
    (seconds per query, results)."""
    secs, results = [], []
    for k, d, a, b in queries:
        t0 = time.perf_counter()
        q = server.submit(k, d, a, b)
        while True:
            fin, _, _ = server.step(stream)
            if q in fin:
                break
        secs.append(time.perf_counter() - t0)
        results.append(server.result(q))
    return np.array(secs), results
