"""Batch-synchronous CPU model of the knapsack search orders of the batched
form: best-first on the heap, breadth-first through the FIFO ring, and the
heap/FIFO switch.  Test infrastructure only: nothing in the library imports
it.

It restates one block's loop of gpuheap_gb300/csrc/search_kernels.cuh
(`run_knapsack`), which follows the reference's models
(artifacts/knapsack/models_pq.cuh:52-137 best-first,
artifacts/knapsack/models_fifo.cuh:13-112 breadth-first,
artifacts/knapsack/models.cuh:102-117 and :210-227 the switch counters):

* a batch is up to `batch` nodes: the best bounds (heap order, nodes whose
  bound no longer beats the incumbent are dropped) or the oldest (FIFO);
* a node whose Dantzig bound beats the incumbent is expanded: the child
  that takes item `level` (if it fits; it raises the incumbent at once) and
  the child that skips it, each kept if its own bound beats the incumbent;
* switch order: heap mode until `counter` batches in a row insert children
  without raising the incumbent, FIFO mode until `counter` batches in a row
  insert children and raise it; at a switch every live node moves over.

The device runs a batch's expansions in parallel, so the order in which
the incumbent rises inside a batch, and which of equal-bound nodes a batch
takes, can differ; the optimum cannot, and switch counts are close to this
model's."""
from fractions import Fraction


def _prepare(w, p):
    """Items by profit/weight, descending (a stable sort, as the host does
    in search.cu), with prefix sums."""
    order = sorted(range(len(w)), key=lambda i: -Fraction(int(p[i]), int(w[i])))
    w = [int(w[i]) for i in order]
    p = [int(p[i]) for i in order]
    W, P = [0], [0]
    for a, b in zip(w, p):
        W.append(W[-1] + a)
        P.append(P[-1] + b)
    return w, p, W, P


def _bound(w, p, W, P, cap, level, profit, weight):
    """Dantzig bound of a node (search_kernels.cuh `knap_bound`: binary
    search for the break item, fractional part floored); -1 if overfull."""
    n = len(w)
    rem = cap - weight
    if rem < 0:
        return -1
    lo, hi = level, n
    while lo < hi:
        mid = (lo + hi + 1) >> 1
        if W[mid] - W[level] <= rem:
            lo = mid
        else:
            hi = mid - 1
    b = profit + (P[lo] - P[level])
    if lo < n:
        b += (rem - (W[lo] - W[level])) * p[lo] // w[lo]
    return b


def search(weights, profits, capacity, order="heap", batch=128, counter=20):
    """Returns (optimum, switches, batches) for one instance."""
    assert order in ("heap", "fifo", "switch")
    w, p, W, P = _prepare(weights, profits)
    n, cap = len(w), int(capacity)
    best = 0
    root = (_bound(w, p, W, P, cap, 0, 0, 0), 0, 0, 0)  # (bound, level, profit, weight)
    mode = 1 if order == "fifo" else 0  # 0 heap, 1 FIFO
    heap, ring = ([], [root]) if mode else ([root], [])
    run = switches = batches = 0
    prev = best
    while True:
        if mode == 0:
            live = sorted((x for x in heap if x[0] > best), key=lambda x: -x[0])
            if not live:
                break
            taken, heap = live[:batch], live[batch:]
        else:
            if not ring:
                break
            taken, ring = ring[:batch], ring[batch:]
        batches += 1
        inserted = 0
        for _, level, profit, weight in taken:
            if _bound(w, p, W, P, cap, level, profit, weight) <= best or level >= n:
                continue
            kids = []
            if weight + w[level] <= cap:
                tp, tw = profit + p[level], weight + w[level]
                best = max(best, tp)
                kids.append((_bound(w, p, W, P, cap, level + 1, tp, tw), level + 1, tp, tw))
            kids.append((_bound(w, p, W, P, cap, level + 1, profit, weight), level + 1, profit, weight))
            for k in kids:
                if k[0] > best:
                    inserted += 1
                    (heap if mode == 0 else ring).append(k)
        if order == "switch":
            raised = best > prev
            run = run + 1 if inserted and (raised if mode == 1 else not raised) else 0
            if run >= counter:
                run = 0
                if mode == 0:
                    ring += sorted((x for x in heap if x[0] > best), key=lambda x: -x[0])
                    heap = []
                else:
                    heap += ring
                    ring = []
                mode ^= 1
                switches += 1
        prev = best
    return best, switches, batches

