"""The batched form's autotuner on CPU: with the batch runner replaced by a
known cost surface, the tuner's search -- batch size x layout on a sample,
then cells per block and the block cap, then the whole-set split and the
runner-up layout -- must land on the surface's minimum, report the timings
it used, and serve a second call from its cache without timing anything."""
import json

import pytest

torch = pytest.importorskip("torch")
from gpuheap_gb300 import batch as gbb  # noqa: E402


def _cost(cfg, n_inst):
    """Seconds for a config: best sample layout is 256 / topdown, best sample
    split 2^19 cells at 16 blocks; on the whole set the 2^20 x 4 split wins
    and the runner-up layout (256 / bottomup) beats the winner there."""
    t = {64: 4.0, 128: 2.0, 256: 1.0, 512: 3.0}[cfg["batch_size"]]
    t += 0.0 if cfg["variant"] == "topdown" else 0.5
    c, mb = cfg["astar_cells_per_block"], cfg["astar_max_blocks"]
    if n_inst <= 8:  # the sample
        t += {1 << 16: 0.4, 1 << 17: 0.3, 1 << 18: 0.2, 1 << 19: 0.1, 1 << 20: 0.25}[c]
        t += {4: 0.3, 8: 0.2, 16: 0.05, 32: 0.15}[mb]
    else:  # the whole set: a different split wins, and bottom-up at 256 is faster
        t = 10.0 + {1 << 18: 0.3, 1 << 19: 0.2, 1 << 20: 0.1}[c] + {4: 0.0, 8: 0.05}[mb]
        if cfg["batch_size"] == 256 and cfg["variant"] == "bottomup":
            t -= 1.0
    return t


@pytest.fixture
def fake_runner(monkeypatch, tmp_path):
    runs = []

    class FakeBatch:
        def __init__(self, insts, **cfg):
            self.cfg, self.n = cfg, len(insts)

        def run(self, mode="graph", stream=None):
            runs.append((dict(self.cfg), self.n))

        def results(self, *a, **k):
            return None

        def close(self):
            pass

    monkeypatch.setattr(gbb, "Batch", FakeBatch)
    monkeypatch.setattr(gbb, "time_run", lambda b, mode, reps=3: _cost(b.cfg, b.n))
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda *a, **k: "fake GB300")
    monkeypatch.setattr(gbb, "_cache_path", lambda: str(tmp_path / "tune.json"))
    return runs


def _instances(n=20):
    return [("knapsack", gbb.gen_knapsack(5 + i, 100 + i)) for i in range(n)]


def test_autotune_sample_stage_finds_the_minimum(fake_runner):
    log = []
    choice = gbb.autotune(_instances(), sample=8, cache=False, log=log.append, full=False)
    assert (choice["batch_size"], choice["variant"]) == (256, "topdown")
    assert (choice["astar_cells_per_block"], choice["astar_max_blocks"]) == (1 << 19, 16)
    assert choice["sample"] == 8 and choice["full_seconds"] is None
    assert choice["sample_seconds"] == pytest.approx(1.0 + 0.1 + 0.05)
    # 8 layouts, then 4 cell sizes and 3 block caps around the best
    assert len(log) == 8 + 4 + 3 and all(e["on"] == "sample" for e in log)


def test_autotune_full_stage_times_the_whole_set(fake_runner):
    log = []
    choice = gbb.autotune(_instances(), sample=8, cache=False, log=log.append, full=True)
    full = [e for e in log if e["on"] == "full"]
    assert len(full) == 3 * 2 + 1  # cells x caps for the best layout, then the runner-up
    assert all(e["batch_size"] == 256 for e in full)
    # the runner-up layout (256 / bottomup) at the winning split wins on the whole set
    assert (choice["batch_size"], choice["variant"]) == (256, "bottomup")
    assert (choice["astar_cells_per_block"], choice["astar_max_blocks"]) == (1 << 20, 4)
    assert choice["full_seconds"] == pytest.approx(10.0 + 0.1 - 1.0)
    whole = [n for _, n in fake_runner if n == 20]
    assert len(whole) >= len(full)


def test_autotune_cache_serves_the_second_call(fake_runner, tmp_path):
    insts = _instances()
    first = gbb.autotune(insts, sample=8, cache=True, full=False)
    n_runs = len(fake_runner)
    with open(tmp_path / "tune.json") as f:
        stored = json.load(f)
    assert list(stored.values()) == [first]
    again = gbb.autotune(insts, sample=8, cache=True, full=False)
    assert again == first and len(fake_runner) == n_runs
    # a different workload signature is tuned afresh
    gbb.autotune(insts[:-1], sample=8, cache=True, full=False)
    assert len(fake_runner) > n_runs
