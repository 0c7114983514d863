"""The served form's host driver on CPU, against a fake server: requests are
admitted only once they have arrived, every result comes back to the query
that asked for it, latency is finish minus arrival, and the plain baseline
runs one query at a time.  Poisson arrivals are seeded and have the asked
rate."""
import time

import numpy as np
import pytest

pytest.importorskip("torch")
from gpuheap_gb300 import serve as gs  # noqa: E402


class FakeServer:
    """Each query needs `work` steps; all admitted queries advance together,
    as slots on the device do.  The result of a query is a function of it."""

    def __init__(self, work):
        self.work = work
        self.left = {}
        self.query = {}
        self.submitted = []
        self.max_in_flight = 0
        self.t0 = time.perf_counter()

    def submit(self, kind, dataset, a, b=0):
        q = len(self.query) + 1000
        self.query[q] = (kind, dataset, a, b)
        self.left[q] = self.work(a)
        self.submitted.append((a, time.perf_counter() - self.t0))
        self.max_in_flight = max(self.max_in_flight, len(self.left))
        return q

    def step(self, stream=None):
        fin = []
        for q in list(self.left):
            self.left[q] -= 1
            if self.left[q] == 0:
                del self.left[q]
                fin.append(q)
        return fin, len(self.left), 0

    def result(self, q):
        kind, d, a, b = self.query[q]
        return 7 * a + b


def test_poisson_arrivals_seeded_and_at_rate():
    a = gs.poisson_arrivals(20000, 500.0, 3)
    assert np.all(np.diff(a) > 0)
    assert np.array_equal(a, gs.poisson_arrivals(20000, 500.0, 3))
    assert not np.array_equal(a, gs.poisson_arrivals(20000, 500.0, 4))
    assert np.mean(np.diff(a)) == pytest.approx(1 / 500.0, rel=0.05)


def test_run_stream_admits_on_arrival_and_maps_results():
    n = 40
    queries = [("sssp", 0, i, i % 3) for i in range(n)]
    arrivals = gs.poisson_arrivals(n, 2000.0, 11)
    srv = FakeServer(lambda a: 1 + a % 5)
    lat, results, makespan, steps = gs.run_stream(srv, queries, arrivals)
    assert results == [7 * i + i % 3 for i in range(n)]
    assert np.all(lat >= 0) and np.all(np.isfinite(lat))
    assert makespan >= arrivals[-1]
    assert steps >= max(1 + i % 5 for i in range(n))
    # no query entered the server before its arrival time
    for a_idx, t in srv.submitted:
        assert t >= arrivals[a_idx] - 1e-6
    assert [a for a, _ in srv.submitted] == list(range(n))


def test_run_plain_runs_one_query_at_a_time():
    queries = [("astar", 1, i, 0) for i in range(6)]
    srv = FakeServer(lambda a: 2 + a)
    secs, results = gs.run_plain(srv, queries)
    assert results == [7 * i for i in range(6)]
    assert srv.max_in_flight == 1 and len(secs) == 6 and np.all(secs >= 0)


def test_run_stream_gives_up_after_its_limit():
    srv = FakeServer(lambda a: 10 ** 9)  # never finishes
    with pytest.raises(RuntimeError, match="did not finish"):
        gs.run_stream(srv, [("sssp", 0, 1, 0)], np.array([0.0]), max_seconds=0.05)
