"""The plain heap-sort autotuner's staged search (gpuheap_gb300/tune.py)
against a fake timer: each stage keeps the best so far, refused
configurations count as infinitely slow, no configuration is timed twice,
and threads outside [32, 1024] are skipped."""
import math

from gpuheap_gb300 import tune


def fake_timer(costs, refuse=()):
    calls = []

    def run(cfg):
        calls.append(dict(cfg))
        key = (cfg["batch_size"], cfg["variant"], cfg["threads"], cfg["grid"], cfg["owner_depth"])
        if key in refuse:
            return math.inf
        t = costs["bs"][cfg["batch_size"]] * costs["var"][cfg["variant"]]
        t *= costs["threads"].get(cfg["threads"], 1.0)
        t *= costs["grid"].get(cfg["grid"], 1.0)
        t *= costs["depth"].get(cfg["owner_depth"], 1.0)
        return t

    return run, calls


def test_stages_pick_the_cheapest_choice_of_each():
    costs = {"bs": {512: 3.0, 1024: 2.0, 2048: 2.5}, "var": {"bottomup": 1.0, "topdown": 1.3},
             "threads": {512: 0.9, 256: 1.2}, "grid": {304: 0.8}, "depth": {0: 1.5, 2: 0.95}}
    run, calls = fake_timer(costs)
    best, t, trials = tune.search(run, 152)
    assert best == {"batch_size": 1024, "variant": "bottomup", "threads": 512, "grid": 304, "owner_depth": 2}
    assert math.isclose(t, 2.0 * 0.9 * 0.8 * 0.95)
    keys = [tuple(sorted(c.items())) for c in calls]
    assert len(keys) == len(set(keys)) == len(trials)


def test_refused_configurations_lose_and_bad_threads_are_skipped():
    costs = {"bs": {512: 1.0, 1024: 2.0}, "var": {"bottomup": 1.0, "topdown": 1.1},
             "threads": {}, "grid": {}, "depth": {}}
    refuse = {(512, "bottomup", 0, 0, -1)}
    run, calls = fake_timer(costs, refuse)
    best, t, _ = tune.search(run, 152, batch_sizes=(512, 1024), keys_per_thread=(0, 1, 8), owner_depths=(-1,))
    assert best["batch_size"] == 512 and best["variant"] == "topdown"
    # 1 key a thread would need 1024 threads at batch 512: allowed; at 2048 it would not be
    assert tune.threads_for(512, 1) == 1024 and tune.threads_for(2048, 1) is None and tune.threads_for(64, 8) is None
    assert all(c["threads"] in (0, 1024, 128) for c in calls)


def test_nothing_runs():
    run = lambda cfg: math.inf  # noqa: E731
    try:
        tune.search(run, 152, batch_sizes=(512,), variants=("bottomup",))
    except RuntimeError:
        return
    raise AssertionError("expected RuntimeError")
