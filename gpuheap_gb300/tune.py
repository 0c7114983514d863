"""Autotuner of the plain heap-sort (gh_heap_sort).

The reference sweeps the plain path's design choices by hand
(artifacts/design_choice/test.sh, sort.cu:85-157): batch size 128-1024 x
threads per block 128..batch size at 128 blocks, then 2-128 blocks at batch
1024.  autotune_sort() searches the same kind of space for this heap, on a
seeded sample of the caller's workload timed on the device, in stages:

  1. batch size x node layout (bottom-up / top-down), other choices
     automatic;
  2. threads per block for the best of stage 1 (automatic, or 2, 4 or 8
     keys a thread in the merges);
  3. blocks (one per SM, half of that, two per SM);
  4. the owner-mode delete's resident depth (automatic, off, 2, 3).

Each stage keeps the best so far; a configuration the heap refuses or that
fails counts as infinitely slow.  Every trial's output is checked against a
device sort of the sample.  The choice is cached per GPU and workload
signature next to the batched tuner's (gpuheap_gb300/_tune_cache.json).
"""
import json
import os

BATCH_SIZES = (512, 1024, 2048)
VARIANTS = ("bottomup", "topdown")
KEYS_PER_THREAD = (0, 2, 4, 8)      # 0: the heap's automatic choice
GRIDS_PER_SM = (1.0, 0.5, 2.0)      # blocks = SMs x this
OWNER_DEPTHS = (-1, 0, 2, 3)        # -1: automatic


def threads_for(batch_size, keys_per_thread):
    """Block threads giving `keys_per_thread` keys a thread in a merge of two
    batches (0: automatic), or None when out of [32, 1024]."""
    if keys_per_thread == 0:
        return 0
    t = 2 * batch_size // keys_per_thread
    return t if 32 <= t <= 1024 else None


def search(run, sms, batch_sizes=BATCH_SIZES, variants=VARIANTS, keys_per_thread=KEYS_PER_THREAD,
           grids_per_sm=GRIDS_PER_SM, owner_depths=OWNER_DEPTHS, log=None):
    """The staged search over configurations; run(cfg) -> seconds (inf when
    the configuration fails).  cfg = {batch_size, variant, threads, grid,
    owner_depth}.  Returns (best cfg, its seconds, every trial)."""
    trials = []

    def trial(cfg):
        key = tuple(sorted(cfg.items()))
        for c, t in trials:
            if tuple(sorted(c.items())) == key:
                return t
        t = run(cfg)
        trials.append((dict(cfg), t))
        if log:
            log(dict(cfg, seconds=t))
        return t

    best, best_t = None, float("inf")
    for bs in batch_sizes:
        for v in variants:
            cfg = dict(batch_size=bs, variant=v, threads=0, grid=0, owner_depth=-1)
            t = trial(cfg)
            if t < best_t:
                best, best_t = cfg, t
    if best is None:
        raise RuntimeError("autotune_sort: no configuration ran")
    for k in keys_per_thread:
        th = threads_for(best["batch_size"], k)
        if th is None:
            continue
        cfg = dict(best, threads=th)
        t = trial(cfg)
        if t < best_t:
            best, best_t = cfg, t
    for g in grids_per_sm:
        blocks = max(2, int(round(sms * g)))
        cfg = dict(best, grid=0 if g == 1.0 else blocks)
        t = trial(cfg)
        if t < best_t:
            best, best_t = cfg, t
    for d in owner_depths:
        cfg = dict(best, owner_depth=d)
        t = trial(cfg)
        if t < best_t:
            best, best_t = cfg, t
    return best, best_t, trials


def _cache_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tune_cache.json")


def autotune_sort(log2n=24, key="u32", dist="uniform", partial_buffer=True, seed=7, reps=2, cache=True, log=None,
                  **space):
    """Picks batch size, layout, block threads, blocks and owner depth for
    gh_heap_sort on 2^log2n seeded keys of `dist` ("uniform" or "zipf").
    Returns the configuration with the sample's seconds per sort.  Keyword
    arguments narrow the search space (see search())."""
    import numpy as np
    import torch

    from . import Heap, HeapError, gen_keys, sort_keys

    dev = torch.cuda.current_device()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    sig = {"what": "sort", "gpu": torch.cuda.get_device_name(dev), "log2n": int(log2n), "key": key, "dist": dist,
           "partial_buffer": bool(partial_buffer), "space": {k: list(v) for k, v in sorted(space.items())}}
    ckey = json.dumps(sig, sort_keys=True)
    path = _cache_path()
    if cache and os.path.exists(path):
        try:
            with open(path) as f:
                got = json.load(f).get(ckey)
            if got:
                return got
        except Exception:
            pass
    n = 1 << int(log2n)
    keys = gen_keys(key, seed, dist, n)
    want = sort_keys(keys, key)
    out = torch.empty_like(keys)

    def run(cfg):
        B = cfg["batch_size"]
        bn = 1
        while bn * B < 2 * n:
            bn <<= 1
        try:
            with Heap(bn, B, key=key, variant=cfg["variant"], partial_buffer=partial_buffer) as h:
                if cfg["threads"]:
                    h.set_block_threads(cfg["threads"])
                if cfg["grid"]:
                    h.set_grid(cfg["grid"])
                h.set_owner_depth(cfg["owner_depth"])
                h.sort(keys, out)  # warm-up
                h.sync()
                if not torch.equal(out, want):
                    return float("inf")
                ts = []
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                for _ in range(reps):
                    ev[0].record()
                    h.sort(keys, out)
                    ev[1].record()
                    h.sync()
                    ts.append(ev[0].elapsed_time(ev[1]) / 1e3)
                return float(np.median(ts))
        except HeapError:
            return float("inf")

    best, best_t, trials = search(run, sms, log=log, **space)
    choice = dict(best, sample_log2n=int(log2n), sample_seconds=round(best_t, 6),
                  sample_mkeys_per_s=round(n / best_t / 1e6, 1), trials=len(trials))
    if cache:
        try:
            data = {}
            if os.path.exists(path):
                with open(path) as f:
                    data = json.load(f)
            data[ckey] = choice
            with open(path, "w") as f:
                json.dump(data, f, indent=1)
        except Exception:
            pass
    return choice
