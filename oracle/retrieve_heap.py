"""Sequential restatement of the reference's retrieving heap
(applications/sssp_longfei_new/heap.cuh): the heap that its SSSP
application drives with insert() and retrieve().  Test infrastructure only:
nothing in the library imports it.

It is a different structure from the four BGPQ variants: nodes are 0-based
(children of i are 2i+1 and 2i+2), the partial buffer is an array of its
own, inserts go top-down only, and retrieve() takes the `size` smallest keys
out of the root and refills the root in place: from the partial buffer, or,
when that holds fewer than `size` keys, from the last node, whose remaining
keys become the new partial buffer; then the root sifts down.

Run by one thread of control, the per-node `is_taken` words only ever move
0 -> 1 -> 0 (an insert marks its target and clears it); the 1 -> 2 -> 3 -> 0
hand-over, where a retrieve takes the target of an insert still in flight,
needs two blocks and is modelled step by step in oracle/lock_model.py
(`retrieve_steal_model`).  Merges follow the reference's merge path with
ties going to the first run (heap/heaputil.cuh:99-158); sorting is by value.

Every step cites the reference line range it restates; the arrays are
numpy, the control flow plain Python.  Pinned by the reference's own runs
(tests/golden/retrieve_ref_cases.npz, tests/test_retrieve_heap_cpu.py):
every returned run and the final nodes, partial buffer and counters.
"""
import numpy as np


def merge_split(a, b):
    """The n smallest of two sorted runs (a first on ties) and the n largest."""
    n = len(a)
    m = np.concatenate([a, b])
    # stable sort keeps a's keys before b's equal keys, as the merge path does
    order = np.argsort(m, kind="stable")
    s = m[order]
    return s[:n].copy(), s[n:].copy()


def next_index(cur, target):
    """The child of `cur` on the path to `target` (0-based nodes), as
    get_next_idx (heap.cuh:50-54): shift target+1 right until it sits one
    level below cur+1."""
    p, q = cur + 1, target + 1
    return (q >> (q.bit_length() - p.bit_length() - 1)) - 1


class RetrievingHeap:
    def __init__(self, batch_num, batch_size, dtype, init_limit):
        self.bn, self.B, self.dt = batch_num, batch_size, dtype
        self.init = dtype(init_limit)
        self.items = np.full(batch_num * batch_size, self.init, dtype)
        self.pb = np.full(batch_size, self.init, dtype)
        self.bc = 0       # curr_batch_count
        self.ps = 0       # curr_pb_size
        self.taken = np.zeros(batch_num, np.int32)

    def node(self, i):
        return self.items[i * self.B:(i + 1) * self.B]

    def set_node(self, i, keys):
        self.items[i * self.B:(i + 1) * self.B] = keys

    def filled(self, keys):
        out = np.full(self.B, self.init, self.dt)
        out[:len(keys)] = keys
        return out

    # ------------------------------------------------------------ insert
    def insert(self, keys):
        """insert(new_items, count) (heap.cuh:272-382); returns False when
        the heap is full (the reference flags need_gc and drops the keys)."""
        keys = np.asarray(keys, self.dt)
        count, B = len(keys), self.B
        assert 0 < count <= B
        if self.bc >= self.bn - 1:
            return False
        if self.ps + count < B:  # case 1: the partial buffer has room (:306-321)
            buf = np.sort(self.filled(np.concatenate([keys, self.pb[:self.ps]])))
            if self.bc == 0:
                self.pb = buf
            else:
                lo, hi = merge_split(buf, self.node(0).copy())
                self.set_node(0, lo)
                self.pb = hi
            self.ps += count
            return True
        # case 2: a full batch forms (:323-336)
        rem = B - count
        buf1 = np.sort(np.concatenate([keys, self.pb[:rem]]))
        rps = self.ps - rem
        buf2 = self.filled(self.pb[rem:self.ps])
        if self.bc == 0:  # 2.1: straight into the root
            lo, hi = merge_split(buf1, buf2)
            self.set_node(0, lo)
            self.pb = hi
            self.bc, self.ps = 1, rps
            return True
        # 2.2: down the path from the root to the new last node (:338-380)
        self.pb = buf2
        self.ps = rps
        target = self.bc
        self.taken[target] = 1
        self.bc += 1
        cur = 0
        while True:
            lo, hi = merge_split(buf1, self.node(cur).copy())
            self.set_node(cur, lo)
            buf1 = hi
            cur = next_index(cur, target)
            if cur == target:
                break
        self.set_node(target, buf1)
        self.taken[target] = 0
        return True

    # ---------------------------------------------------------- retrieve
    def retrieve(self, size):
        """retrieve(ret, *size) (heap.cuh:79-270): the `size` smallest keys
        (fewer when fewer are held), ascending."""
        B = self.B
        size = min(size, B)
        if self.bc == 0:  # case 1: from the partial buffer (:98-114)
            n = min(size, self.ps)
            out = self.pb[:n].copy()
            rest = self.pb[n:self.ps].copy()
            self.pb[:len(rest)] = rest
            self.ps -= n
            return out
        out = self.node(0)[:size].copy()
        rem = B - size
        if self.bc == 1:  # case 2: only the root (:119-145)
            root_rest = self.node(0)[size:].copy()
            if self.ps >= size:
                self.set_node(0, np.concatenate([root_rest, self.pb[:size]]))
                rest = self.pb[size:self.ps].copy()
                self.pb[:len(rest)] = rest
                self.ps -= size
            else:
                keep = np.concatenate([root_rest, self.pb[:self.ps]])
                self.pb[:len(keep)] = keep
                self.bc = 0
                self.ps = len(keep)
            return out
        # case 3: refill from the partial buffer, then the last node (:147-199)
        buf1 = np.empty(B, self.dt)
        buf1[:rem] = self.node(0)[size:]
        if self.ps >= size:
            buf1[rem:] = self.pb[:size]
            buf2 = self.filled(self.pb[size:self.ps])
            self.ps -= size
        else:
            buf1[rem:rem + self.ps] = self.pb[:self.ps]
            gap = size - self.ps
            self.bc -= 1
            last = self.bc
            assert self.taken[last] == 0  # one thread of control: no insert in flight
            lastkeys = self.node(last).copy()
            buf1[B - gap:] = lastkeys[:gap]
            buf2 = self.filled(lastkeys[gap:])
            buf1 = np.sort(buf1)
            buf1, buf2 = merge_split(buf1, buf2)
            self.ps = B - gap
        self.pb = buf2.copy()
        # sift the new root down (:201-268)
        cur = 0
        while True:
            l, r = 2 * cur + 1, 2 * cur + 2
            left = l < self.bn and self.bc > l and self.taken[l] == 0
            right = r < self.bn and self.bc > r and self.taken[r] == 0
            if not left and not right:
                self.set_node(cur, buf1)
                break
            if left and not right:
                lo, buf1 = merge_split(buf1, self.node(l).copy())
                self.set_node(cur, lo)
                cur = l
            elif right and not left:
                lo, buf1 = merge_split(buf1, self.node(r).copy())
                self.set_node(cur, lo)
                cur = r
            else:
                a, b = self.node(l).copy(), self.node(r).copy()
                if a[-1] <= b[-1]:
                    a, b = merge_split(a, b)
                    self.set_node(r, b)
                    lo, buf1 = merge_split(buf1, a)
                    self.set_node(cur, lo)
                    cur = l
                else:
                    lo2, hi2 = merge_split(a, b)
                    self.set_node(l, hi2)
                    lo, buf1 = merge_split(buf1, lo2)
                    self.set_node(cur, lo)
                    cur = r
        return out

    def state(self):
        """(valid nodes, valid partial buffer, [batch count, pb size])."""
        return (self.items[:self.bc * self.B].copy(), self.pb[:self.ps].copy(),
                np.array([self.bc, self.ps], np.int32))
