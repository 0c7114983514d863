"""SSSP with the queue on the GPU, bit-exact against the CPU Dijkstra oracle."""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402
from gpuheap_gb300 import sssp as gsssp  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield


def sources_of(graph_host, k, seed):
    rowptr = graph_host[0]
    deg = np.diff(rowptr)
    rng = np.random.default_rng(seed)
    return rng.choice(np.nonzero(deg)[0], size=k, replace=False)


@pytest.mark.parametrize("variant", ["bottomup", "topdown"])
@pytest.mark.parametrize("scale,B", [(12, 256), (14, 1024), (16, 1024)])
def test_sssp_matches_dijkstra(variant, scale, B):
    g = gsssp.rmat_graph(scale, 16, seed=scale * 7 + 1)
    host = g.host()
    heap = gsssp.make_heap(g, batch_size=B, variant=variant)
    srcs = sources_of(host, 4, scale)
    want = pyoracle.dijkstra(*host, srcs, threads=8)
    for i, s in enumerate(srcs):
        dist, st = gsssp.sssp(heap, g, int(s))
        got = dist.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, want[i]), f"source {s}"
        assert st["keys_taken"] >= st["keys_inserted"] - 0 and st["keys_inserted"] >= 1
    heap.close()


def test_sssp_isolated_source_and_graph_shape():
    g = gsssp.rmat_graph(10, 8, seed=3)
    rowptr, col, w = g.host()
    assert rowptr[-1] == col.size and np.all(np.diff(rowptr) >= 0)
    assert w.min() >= 1 and w.max() <= 1000
    # symmetric: every edge has its reverse with the same weight
    src = np.repeat(np.arange(g.n), np.diff(rowptr))
    fwd = set(zip(src.tolist(), col.tolist(), w.tolist()))
    assert all((d, s, ww) in fwd for s, d, ww in list(fwd)[:2000])
    heap = gsssp.make_heap(g, batch_size=256)
    iso = np.nonzero(np.diff(rowptr) == 0)[0]
    if iso.size:
        dist, _ = gsssp.sssp(heap, g, int(iso[0]))
        d = dist.cpu().numpy().view(np.uint32)
        assert d[iso[0]] == 0 and np.sum(d != 0xFFFFFFFF) == 1
    heap.close()
