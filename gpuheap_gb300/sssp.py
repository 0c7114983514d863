"""Single-source shortest paths with the batched priority queue.

rmat_graph() builds the synthetic R-MAT graph of the SSSP workload on the
device (edges from gh_rmat_edges, symmetrised as
applications/sssp_longfei_new/main.cu:46-49 does, self loops dropped, CSR by
a key sort -- torch is only plumbing here); sssp() runs gh_sssp, the
heap-driven SSSP kernel.
"""
import ctypes

from . import Heap, _check, lib


class Graph:
    """CSR graph on the device: rowptr (n+1, int64), col (int32), w (int32 bits of u32)."""

    def __init__(self, n, rowptr, col, w):
        self.n = int(n)
        self.rowptr = rowptr
        self.col = col
        self.w = w

    @property
    def m(self):
        return int(self.col.numel())

    def host(self):
        """numpy copies (rowptr int64, col int32, w uint32)."""
        import numpy as np
        return (self.rowptr.cpu().numpy(), self.col.cpu().numpy(), self.w.cpu().numpy().view(np.uint32))


def rmat_graph(scale, edge_factor=16, seed=1, a=0.57, b=0.19, c=0.19, max_weight=1000, device="cuda"):
    """R-MAT graph of 2^scale vertices and edge_factor * 2^scale generated
    edges (weights uniform in [1, max_weight]), symmetrised, as CSR."""
    import torch
    n = 1 << scale
    m = edge_factor * n
    src = torch.empty(m, dtype=torch.int32, device=device)
    dst = torch.empty(m, dtype=torch.int32, device=device)
    w = torch.empty(m, dtype=torch.int32, device=device)
    _check(lib().gh_rmat_edges(scale, m, a, b, c, seed, max_weight, src.data_ptr(), dst.data_ptr(), w.data_ptr(),
                               torch.cuda.current_stream().cuda_stream), "rmat_edges")
    keep = src != dst
    s2 = torch.cat([src[keep], dst[keep]]).to(torch.int64)
    d2 = torch.cat([dst[keep], src[keep]]).to(torch.int64)
    w2 = torch.cat([w[keep], w[keep]])
    order = torch.argsort(s2 * n + d2)
    s2, d2, w2 = s2[order], d2[order], w2[order]
    rowptr = torch.zeros(n + 1, dtype=torch.int64, device=device)
    rowptr[1:] = torch.cumsum(torch.bincount(s2, minlength=n), 0)
    return Graph(n, rowptr, d2.to(torch.int32).contiguous(), w2.contiguous())


# SSSP runs fastest with large batches on few blocks: every block that takes
# a batch at the same time takes keys farther from the minimum, so vertices
# are expanded again later, and all blocks contend on one root.  On GB300,
# R-MAT scales 18-22: batch 2048 on 24 blocks beat every other point of a
# sweep over batch {1024, 2048} x blocks {6 .. 152} (scale 22: 109 ms per
# source on 24 blocks, 341 ms at batch 1024 on 152).
SSSP_BATCH, SSSP_BLOCKS = 2048, 24


def make_heap(graph, batch_size=SSSP_BATCH, variant="bottomup", capacity_keys=None, blocks=SSSP_BLOCKS):
    """A u64-key heap (partial buffer on) large enough for SSSP on `graph`,
    running SSSP on `blocks` blocks (0 = one per SM)."""
    keys = capacity_keys or max(4 * graph.n, graph.m // 2, 1 << 16)
    bn = 1
    while bn * batch_size < keys:
        bn <<= 1
    h = Heap(bn, batch_size, key="u64", variant=variant, partial_buffer=True)
    if blocks:
        h.set_grid(blocks)
    return h


def sssp(heap, graph, source, dist=None, stream=None):
    """Distances from `source` (u32 bits in an int32 tensor; UINT32_MAX =
    unreachable) and {keys_taken, edges_scanned, keys_inserted}."""
    import torch
    if dist is None:
        dist = torch.empty(graph.n, dtype=torch.int32, device=graph.col.device)
    stats = (ctypes.c_ulonglong * 3)()
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    _check(lib().gh_sssp(heap._h, graph.n, graph.rowptr.data_ptr(), graph.col.data_ptr(), graph.w.data_ptr(),
                         int(source), dist.data_ptr(), s, stats), "sssp")
    return dist, {"keys_taken": stats[0], "edges_scanned": stats[1], "keys_inserted": stats[2]}


def sssp_retrieve(graph, source, batch_size=256, chunk=32, blocks=32, capacity_keys=0, dist=None, stream=None):
    """SSSP through the retrieving heap with the auxiliary buffer
    (gh_sssp_retrieve; the reference's ssspKernel,
    applications/sssp_longfei_new/sssp.cu:19-132).  Returns (distances as
    u32 bits in an int32 tensor, {keys_taken, edges, keys_inserted,
    handovers})."""
    import torch
    if dist is None:
        dist = torch.empty(graph.n, dtype=torch.int32, device=graph.col.device)
    stats = (ctypes.c_ulonglong * 4)()
    s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    _check(lib().gh_sssp_retrieve(graph.n, graph.rowptr.data_ptr(), graph.col.data_ptr(), graph.w.data_ptr(),
                                  int(source), dist.data_ptr(), int(batch_size), int(chunk), int(blocks),
                                  int(capacity_keys), s, stats), "sssp_retrieve")
    return dist, {"keys_taken": stats[0], "edges": stats[1], "keys_inserted": stats[2], "handovers": stats[3]}
