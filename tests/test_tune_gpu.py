"""The plain heap-sort autotuner on the GPU (gpuheap_gb300/tune.py): on a
small sample over a narrowed space it returns a configuration the heap
accepts, and a heap-sort with that configuration is exact."""
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
import gpuheap_gb300 as gh  # noqa: E402
from gpuheap_gb300 import tune  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda(ghlib):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield


@pytest.mark.parametrize("key", ["u32", "u64"])
def test_autotune_sort_small(key):
    seen = []
    cfg = tune.autotune_sort(log2n=18, key=key, cache=False, reps=1, log=seen.append, batch_sizes=(512, 1024),
                             variants=("bottomup", "topdown"), keys_per_thread=(0, 4), grids_per_sm=(1.0, 0.5),
                             owner_depths=(-1, 0))
    assert cfg["sample_seconds"] > 0 and cfg["trials"] == len(seen) >= 6
    assert all(s["seconds"] > 0 for s in seen)
    n = 1 << 19
    keys = gh.gen_keys(key, 99, "uniform", n)
    out = torch.empty_like(keys)
    bn = 1
    while bn * cfg["batch_size"] < 2 * n:
        bn <<= 1
    with gh.Heap(bn, cfg["batch_size"], key=key, variant=cfg["variant"]) as h:
        if cfg["threads"]:
            h.set_block_threads(cfg["threads"])
        if cfg["grid"]:
            h.set_grid(cfg["grid"])
        h.set_owner_depth(cfg["owner_depth"])
        h.sort(keys, out)
        h.sync()
    assert torch.equal(out, gh.sort_keys(keys, key))
