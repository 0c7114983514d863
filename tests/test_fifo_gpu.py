"""The device FIFO buffer on the GPU, through the C ABI.

One block: every push / pop replays exactly against the sequential
restatement of the reference's Buffer<K> (oracle FifoModel), output and
positions.  Many blocks: the reference's own test (bufferTest.cu:13-175)
checks that what comes out is what went in; here, in addition, each
insertToBuffer piece must come out whole and in order, and keys pushed by
one block before a concurrent run must come out first, in their order.
"""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402
from gpuheap_gb300.fifo import Fifo  # noqa: E402

NP = {"u32": np.uint32, "i32": np.int32, "u64": np.uint64}
TORCH = {"u32": torch.int32, "i32": torch.int32, "u64": torch.int64}


@pytest.fixture(scope="module", autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield


def dev(a, key):
    a = np.ascontiguousarray(a, NP[key])
    view = a.view(np.int64 if key == "u64" else np.int32)
    return torch.from_numpy(view.copy()).cuda()


def host(t, key):
    return t.cpu().numpy().view(NP[key])


def distinct_keys(rng, n, key):
    hi = {"u32": 2**32 - 1, "i32": 2**31 - 1, "u64": 2**63}[key]
    lo = -(2**31) if key == "i32" else 0
    k = rng.choice(np.arange(0, 4 * n + 16), size=n, replace=False).astype(np.int64) + lo
    assert k.max() < hi
    return k.astype(NP[key])


@pytest.mark.parametrize("key", ["u32", "i32", "u64"])
@pytest.mark.parametrize("capacity", [64, 1000, 4096])
def test_single_block_replay(key, capacity):
    """Random pushes and pops by one block equal the sequential model,
    through many laps of a small ring."""
    rng = np.random.default_rng(capacity + len(key))
    model = pyoracle.FifoModel(capacity, NP[key])
    with Fifo(capacity, key) as f:
        assert f.capacity == model.capacity
        f.set_launch(blocks=1, threads=128)
        next_key = 0
        for step in range(60):
            held = model.end - model.begin
            whole = rng.random() < 0.3  # chunk 0: one reservation / claim for the call
            if rng.random() < 0.55:
                n = int(rng.integers(0, f.capacity - held + 1))
                chunk = 0 if whole else int(rng.integers(1, min(f.capacity, 300) + 1))
                keys = (np.arange(next_key, next_key + n) * 7 + 3).astype(NP[key])
                next_key += n
                model.push(keys, chunk or max(n, 1))
                if n:
                    f.push(dev(keys, key), chunk=chunk)
                else:
                    f.push(torch.empty(0, dtype=TORCH[key], device="cuda"), n=0, chunk=chunk)
            else:
                max_keys = int(rng.integers(0, f.capacity + 5))
                chunk = 0 if whole else int(rng.integers(1, 400))
                want = model.pop(max_keys, chunk or max(max_keys, 1))
                out = torch.full((max(max_keys, 1),), -1, dtype=TORCH[key], device="cuda")
                got_n = f.pop(out, max_keys=max_keys, chunk=chunk)
                assert got_n == len(want), (step, got_n, len(want))
                assert np.array_equal(host(out, key)[:got_n], want), step
            assert f.positions() == model.positions(), step
        assert f.count() == model.end - model.begin


@pytest.mark.parametrize("key", ["u32", "u64"])
@pytest.mark.parametrize("chunk", [1, 100, 1024, 4096])
def test_many_blocks_pieces_whole(key, chunk):
    """Many pushing blocks then many popping blocks: a permutation in which
    every piece is whole and in order."""
    rng = np.random.default_rng(chunk)
    n = 200_000 if chunk > 1 else 20_000
    keys = distinct_keys(rng, n, key)
    with Fifo(1 << 18, key) as f:
        f.push(dev(keys, key), chunk=chunk)
        out = torch.empty(n + 10, dtype=TORCH[key], device="cuda")
        got = f.pop(out, chunk=chunk if chunk > 1 else 333)
        assert got == n
        assert pyoracle.fifo_pieces_ok(keys, host(out, key)[:n], pyoracle.fifo_piece_starts(n, chunk, False))
        assert f.positions() == (n, n, n, n)
        assert f.pop(out) == 0


@pytest.mark.parametrize("key", ["u32", "i32", "u64"])
@pytest.mark.parametrize("n,capacity", [(1, 1), (1000, 1024), (3_000_001, 1 << 22), (1 << 24, 1 << 24)])
def test_whole_call_exact_order(key, n, capacity):
    """chunk 0: one reservation per push and one claim per pop -- the grid
    copies, and the keys come out exactly in input order, also across a wrap."""
    rng = np.random.default_rng(n)
    keys = distinct_keys(rng, n, key) if n < 4_000_000 else np.arange(n, dtype=NP[key])
    with Fifo(capacity, key) as f:
        out = torch.empty(n, dtype=TORCH[key], device="cuda")
        pre = min(n // 3 + 1, f.capacity) if n > 1 else 0   # move the ring's start off zero
        if pre:
            f.push(dev(keys[:pre], key))
            assert f.pop(out, max_keys=pre) == pre
        f.push(dev(keys, key))
        assert f.pop(out) == n
        assert np.array_equal(host(out, key), keys)
        assert f.positions() == (pre + n,) * 4
        assert f.pop(out) == 0


@pytest.mark.parametrize("key", ["u32", "i32"])
@pytest.mark.parametrize("array_num,chunk,blocks", [(1 << 20, 1024, 0), (100_000, 512, 8), (300_000, 96, 64)])
def test_reference_concurrent_flow(key, array_num, chunk, blocks):
    """bufferTest.cu's flow: insert array_num keys, then half the blocks
    insert array_num more (each piece as a third and the rest) while the
    other half take array_num, then take the rest.  The ring holds exactly
    array_num keys' worth (rounded to a power of two), so pushers wait for
    room."""
    rng = np.random.default_rng(array_num)
    first = distinct_keys(rng, 2 * array_num, key)
    second = first[array_num:]
    first = first[:array_num]
    with Fifo(array_num, key) as f:
        f.set_launch(blocks=1, threads=256)
        f.push(dev(first, key), chunk=chunk)  # one block: ring order = input order
        f.set_launch(blocks=blocks, threads=256)
        out = torch.empty(array_num, dtype=TORCH[key], device="cuda")
        got = f.concurrent(dev(second, key), out, chunk=chunk, max_keys=array_num)
        assert got == array_num
        assert np.array_equal(host(out, key), first), "keys held before the run come out first, in order"
        rest = torch.empty(array_num, dtype=TORCH[key], device="cuda")
        assert f.pop(rest, chunk=chunk) == array_num
        assert pyoracle.fifo_pieces_ok(second, host(rest, key), pyoracle.fifo_piece_starts(array_num, chunk, True))
        assert f.positions() == (2 * array_num,) * 4


@pytest.mark.parametrize("capacity,chunk", [(64, 16), (64, 64), (256, 7)])
def test_concurrent_many_laps(capacity, chunk):
    """A tiny ring, lapped thousands of times by concurrent pushers and poppers."""
    rng = np.random.default_rng(capacity * chunk)
    n = 100_000
    keys = distinct_keys(rng, n, "u32")
    with Fifo(capacity, "u32") as f:
        f.set_launch(blocks=16, threads=64)
        out = torch.empty(n, dtype=torch.int32, device="cuda")
        assert f.concurrent(dev(keys, "u32"), out, chunk=chunk, max_keys=n) == n
        assert pyoracle.fifo_pieces_ok(keys, host(out, "u32"), pyoracle.fifo_piece_starts(n, chunk, True))
        assert f.positions() == (n,) * 4


def test_concurrent_partial_take():
    """The poppers stop at max_keys; the rest stays in the ring, in order."""
    rng = np.random.default_rng(5)
    n = 50_000
    keys = distinct_keys(rng, n, "u64")
    with Fifo(1 << 16, "u64") as f:
        f.set_launch(blocks=1, threads=128)
        out = torch.empty(n, dtype=torch.int64, device="cuda")
        # one pushing and one popping block: FIFO order = input order
        f.set_launch(blocks=2, threads=128)
        assert f.concurrent(dev(keys, "u64"), out, chunk=1000, max_keys=12_345) == 12_345
        assert np.array_equal(host(out, "u64")[:12_345], keys[:12_345])
        rest = torch.empty(n, dtype=torch.int64, device="cuda")
        assert f.pop(rest) == n - 12_345
        assert np.array_equal(host(rest, "u64")[:n - 12_345], keys[12_345:])


def test_edges_and_errors():
    with Fifo(100, "u32") as f:
        assert f.capacity == 128
        out = torch.empty(16, dtype=torch.int32, device="cuda")
        assert f.pop(out) == 0                      # empty
        assert f.pop(out, max_keys=0) == 0
        keys = dev(np.arange(128), "u32")
        f.push(keys)                                # exactly full
        assert f.count() == 128
        with pytest.raises(gh.HeapError) as e:      # one more key cannot fit
            f.push(keys, n=1)
        assert e.value.status == gh.GH_ERR_CAPACITY
        with pytest.raises(gh.HeapError) as e:      # chunk above the ring
            f.push(keys, n=0, chunk=129)
        assert e.value.status == gh.GH_ERR_INVALID
        with pytest.raises(gh.HeapError) as e:      # would wait for keys that never come
            f.concurrent(keys, torch.empty(300, dtype=torch.int32, device="cuda"), n=10, max_keys=200)
        assert e.value.status == gh.GH_ERR_INVALID
        assert f.pop(out, chunk=5) == 16
        assert np.array_equal(host(out, "u32"), np.arange(16))
        assert f.positions() == (16, 16, 128, 128)
        f.reset()
        assert f.positions() == (0, 0, 0, 0)
        view = f.device_view()
        assert len(view) == gh.lib().gh_fifo_view_bytes()
        ptrs = np.frombuffer(view[:24], np.uint64)
        assert ptrs[2] == 128                       # items, state, capacity


def test_timeout_on_unpublished_reservation():
    """A reservation that is never published holds up every later push; the
    bounded wait turns it into GH_ERR_TIMEOUT, later calls get GH_ERR_STATE
    until reset."""
    with Fifo(1024, "u32") as f:
        f.set_timeout(0.05)
        f.set_launch(blocks=1, threads=64)
        keys = dev(np.arange(10), "u32")
        f.inject_reservation(5)
        f.push(keys)
        with pytest.raises(gh.HeapError) as e:
            f.count()
        assert e.value.status == gh.GH_ERR_TIMEOUT
        assert f.info()["err_site"] == 2            # waiting to publish
        with pytest.raises(gh.HeapError) as e:
            f.pop(torch.empty(10, dtype=torch.int32, device="cuda"))
        assert e.value.status == gh.GH_ERR_STATE
        f.reset()
        f.push(keys)
        out = torch.empty(10, dtype=torch.int32, device="cuda")
        assert f.pop(out) == 10
        assert np.array_equal(host(out, "u32"), np.arange(10))
