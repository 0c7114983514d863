"""The oracle's restatement of the reference's retrieving heap
(oracle/retrieve_heap.py; applications/sssp_longfei_new/heap.cuh) replayed
over the reference's own insert / retrieve sequences
(tests/golden/retrieve_ref_cases.npz): every returned run and count, and the
heap each sequence leaves (valid nodes, partial buffer, counters), bit for
bit.  Also the path index of the top-down insert against a direct walk."""
import numpy as np
import pytest

import golden_cases
from oracle.retrieve_heap import RetrievingHeap, next_index

NP = {"u32": np.uint32, "u64": np.uint64}
INIT = {"u32": 0xFFFFFFFF, "u64": 2**64 - 1}


def replay(c):
    h = RetrievingHeap(c["batch_num"], c["batch_size"], NP[c["key"]], INIT[c["key"]])
    pos, runs, taken = 0, [], []
    for op in c["ops"]:
        if op > 0:
            assert h.insert(c["keys"][pos:pos + op])
            pos += op
        else:
            got = h.retrieve(-int(op))
            runs.append(got)
            taken.append(len(got))
    return h, np.concatenate(runs) if runs else np.zeros(0, NP[c["key"]]), np.asarray(taken, np.int32)


@pytest.mark.parametrize("i", range(len(golden_cases.retrieve_meta())))
def test_model_matches_the_reference_bit_for_bit(i):
    c = golden_cases.retrieve_case(i)
    h, runs, taken = replay(c)
    assert np.array_equal(taken, c["taken"])
    assert np.array_equal(runs, c["runs"])
    nodes, pb, counters = h.state()
    assert np.array_equal(counters, c["final_counters"])
    assert np.array_equal(nodes, c["final_nodes"])
    assert np.array_equal(pb, c["final_pb"])


def test_path_index_walks_down_to_the_target():
    for target in range(1, 2048):
        path, cur = [], 0
        while cur != target:
            cur = next_index(cur, target)
            path.append(cur)
        # each step goes one level down to a child, ending at the target
        want, t = [], target
        while t > 0:
            want.append(t)
            t = (t - 1) // 2
        assert path == want[::-1]
