"""The heap's block primitives on their own against numpy: the merge of two
sorted batches (every insert and sift step's merge path, and the owner-mode
delete's warp windows) and the bitonic sort of an insert batch.

Grid: the reference's local_test/merge_path/test.sh:5-16 (batch 32..2048 x
block 32..min(batch, 1024)), where the merge path's keys per thread stay in
1..16; every key type; keys with many ties.  Bar: bit-exact."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402

KIND = {"u32": 0, "i32": 1, "u64": 2}
NP = {"u32": np.uint32, "i32": np.int32, "u64": np.uint64}
STORE = {"u32": np.int32, "i32": np.int32, "u64": np.int64}
GRID = [(b, t) for b in (32, 64, 128, 256, 512, 1024, 2048) for t in (32, 64, 128, 256, 512, 1024) if t <= min(b, 1024)]


@pytest.fixture(autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)


def keys(rng, key, n, ties):
    hi = 40 if ties else (2**31 - 1 if key == "i32" else 2**32 - 2)
    v = rng.integers(-hi if key == "i32" and ties else 0, hi, n)
    if key == "u64":
        v = (v.astype(np.uint64) << np.uint64(32)) | rng.integers(0, 2**32, n).astype(np.uint64)
    return np.sort(v.astype(NP[key]))


def dev(a, key):
    return torch.from_numpy(np.ascontiguousarray(a).view(STORE[key])).cuda()


def host(t, key):
    return t.cpu().numpy().view(NP[key])


def merge(key, method, a, b, threads):
    n = a.size
    lo = torch.zeros(n, dtype=torch.int64 if key == "u64" else torch.int32, device="cuda")
    hi = torch.zeros_like(lo)
    da, db = dev(a, key), dev(b, key)
    st = gh.lib().gh_merge_batches(KIND[key], method, ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(db.data_ptr()),
                                   n, ctypes.c_void_p(lo.data_ptr()), ctypes.c_void_p(hi.data_ptr()), threads, None)
    assert st == 0, gh.lib().gh_status_string(st)
    torch.cuda.synchronize()
    return host(lo, key), host(hi, key)


@pytest.mark.parametrize("B,threads", [g for g in GRID if 2 * g[0] // g[1] <= 16])
@pytest.mark.parametrize("key", ["u32", "i32", "u64"])
def test_merge_path_grid(B, threads, key):
    rng = np.random.default_rng(B * 7 + threads)
    for ties in (False, True):
        a, b = keys(rng, key, B, ties), keys(rng, key, B, ties)
        lo, hi = merge(key, 0, a, b, threads)
        want = np.sort(np.concatenate([a, b]))
        assert np.array_equal(lo, want[:B]) and np.array_equal(hi, want[B:]), (B, threads, ties)


@pytest.mark.parametrize("B", [256, 512, 1024, 2048, 4096])
@pytest.mark.parametrize("key", ["u32", "i32", "u64"])
@pytest.mark.parametrize("threads", [32, 256, 1024])
def test_warp_window_merge(B, key, threads):
    if 2 * B < (512 if key == "u64" else 1024):
        pytest.skip("smaller than one window")
    rng = np.random.default_rng(B + threads)
    for ties in (False, True):
        a, b = keys(rng, key, B, ties), keys(rng, key, B, ties)
        lo, hi = merge(key, 1, a, b, threads)
        want = np.sort(np.concatenate([a, b]))
        assert np.array_equal(lo, want[:B]) and np.array_equal(hi, want[B:]), (B, threads, ties)


@pytest.mark.parametrize("B,threads", GRID)
@pytest.mark.parametrize("key", ["u32", "u64"])
def test_bitonic_sort_grid(B, threads, key):
    rng = np.random.default_rng(B + 3 * threads)
    for ties in (False, True):
        v = rng.permutation(keys(rng, key, B, ties))
        out = torch.zeros(B, dtype=torch.int64 if key == "u64" else torch.int32, device="cuda")
        d = dev(v, key)
        st = gh.lib().gh_sort_batch(KIND[key], ctypes.c_void_p(d.data_ptr()), B, ctypes.c_void_p(out.data_ptr()),
                                    threads, None)
        assert st == 0
        torch.cuda.synchronize()
        assert np.array_equal(host(out, key), np.sort(v)), (B, threads, ties)
