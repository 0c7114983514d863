"""Randomised properties of the oracle's Heap<K> model, beyond the golden
sequences: over seeded random mixes of insertions and deletions, for every
variant, key type and a tie-heavy key set, each deleteRoot returns exactly
the smallest keys present -- a whole batch while full nodes remain, the
partial buffer after that -- and checkInsertHeap accepts the model's memory
after every operation."""
import numpy as np
import pytest

from oracle import pyoracle

LIMIT = {"u32": (0, 2**32 - 1), "u64": (0, 2**64 - 1), "i32": (-(2**31), 2**31 - 1)}


def _keys(rng, key, n, ties):
    lo, hi = LIMIT[key]  # hi is init_limits: keys stay strictly below it
    dt = pyoracle.DTYPES[key]
    if ties:
        return rng.integers(lo, lo + 12, n, dtype=dt)
    if key == "u64":
        return rng.integers(0, 2**63, n, dtype=np.uint64)
    return rng.integers(lo, hi, n, dtype=dt)


@pytest.mark.parametrize("key", ["u32", "u64", "i32"])
@pytest.mark.parametrize("variant,pb", [("topdown", True), ("topdown", False), ("bottomup", True),
                                        ("bottomup", False)])
def test_model_is_a_priority_queue_on_random_mixes(variant, pb, key):
    for seed in range(40):
        rng = np.random.default_rng(7000 + seed)
        B = [16, 32, 64][seed % 3]
        ties = seed % 4 == 0
        nb = int(rng.integers(6, 16))
        n = nb * B
        bn = 1
        while bn * B < 2 * n:
            bn <<= 1
        m = pyoracle.Model(key, variant, pb, bn, B)
        keys = _keys(rng, key, n, ties)
        out = np.zeros(n + 2 * B, pyoracle.DTYPES[key])
        present = np.empty(0, keys.dtype)
        pos = cursor = 0
        while pos < n or present.size:
            if pos < n and (present.size == 0 or rng.random() < 0.6):
                # heaps without the partial buffer take full batches only
                s = B if not pb else int(rng.integers(1, B + 1))
                s = min(s, n - pos)
                if not pb and s < B:
                    s = n - pos  # n is a multiple of B, so this is a full batch
                assert m.insert(keys[pos:pos + s]) == 0
                present = np.sort(np.concatenate([present, keys[pos:pos + s]]))
                pos += s
            else:
                items, counters = m.state()
                bc, ps = int(counters[0]), int(counters[1])
                sz = m.delete(out)
                assert sz == (B if bc > 0 else ps), (seed, bc, ps, sz)
                assert np.array_equal(out[cursor:cursor + sz], present[:sz]), seed
                present = present[sz:]
                cursor += sz
            items, counters = m.state()
            assert int(counters[0]) * B + int(counters[1]) == present.size
            ok = pyoracle.check_heap(variant, items, None, B, int(counters[0]), int(counters[1]))
            assert ok, (seed, ok)
        assert cursor == n
        assert np.array_equal(np.sort(out[:n]), np.sort(keys))  # every key out once
