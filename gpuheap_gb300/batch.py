"""Batched searches: many independent grid A* and 0/1 knapsack instances of
uneven size, each on its own heap, in one persistent launch (gh_batch_*).

workload() draws the synthetic mix (grids with sides log-uniform in
[256, 4096], 20 % obstacles, cell costs 1-9; knapsacks with 100-1000 items,
weights 1-1000, profit = weight + U(0, 100), capacity half the total
weight).  Batch wraps the C ABI; autotune() picks batch size, block threads,
node layout and A* blocks per instance by timing candidates on a sample and
caches the choice.
"""
import ctypes
import json
import os
import time

import numpy as np

from . import _check, _I, _LL, _VP, lib

ASTAR, KNAPSACK = 0, 1
PERSISTENT, GRAPH, PLAIN = 0, 1, 2
_MODES = {"persistent": PERSISTENT, "graph": GRAPH, "plain": PLAIN}
_VARIANTS = {"topdown": 0, "bottomup": 1}
KNAPSACK_ORDERS = {"heap": 0, "fifo": 1, "switch": 2}


def gen_grid(side, seed, obstacle_per_mille=200, height=None):
    """Seeded (height, side) uint8 cost grid through gh_gen_grid (0 = obstacle)."""
    h = side if height is None else height
    out = np.empty((h, side), np.uint8)
    _check(lib().gh_gen_grid(side, h, seed, obstacle_per_mille, out.ctypes.data, os.cpu_count() or 1), "gen_grid")
    return out


def gen_knapsack(n, seed):
    """(weights, profits, capacity): weights 1-1000, profit = weight + U(0, 100),
    capacity = floor(total weight / 2)."""
    rng = np.random.default_rng(seed)
    w = rng.integers(1, 1001, n).astype(np.int32)
    p = (w + rng.integers(0, 101, n)).astype(np.int32)
    return w, p, int(w.sum()) // 2


def workload(count=1024, seed=2026, astar_share=0.5, min_side=256, max_side=4096, min_items=100, max_items=1000):
    """The batched mix: a list of ("astar", grid) and ("knapsack", (w, p, cap)),
    instance i drawn from (seed, i)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        inst_seed = int(rng.integers(1 << 62))
        if rng.random() < astar_share:
            u = rng.random()
            side = int(round(min_side * (max_side / min_side) ** u))
            out.append(("astar", gen_grid(side, inst_seed)))
        else:
            n = int(rng.integers(min_items, max_items + 1))
            out.append(("knapsack", gen_knapsack(n, inst_seed)))
    return out


class Batch:
    """A set of searches uploaded once and run any number of times."""

    def __init__(self, instances, batch_size=256, variant="bottomup", block_threads=0, astar_cells_per_block=1 << 18,
                 astar_max_blocks=8, timeout=2.0, stream=None, knapsack_order="heap", switch_counter=20):
        h = _VP()
        _check(lib().gh_batch_create(ctypes.byref(h), batch_size, _VARIANTS[variant], block_threads), "batch_create")
        self._h = h
        self.batch_size, self.variant, self.block_threads = batch_size, variant, block_threads
        self.kinds = []
        try:
            _check(lib().gh_batch_set_timeout(h, float(timeout)), "batch_set_timeout")
            _check(lib().gh_batch_set_astar_blocks(h, int(astar_cells_per_block), int(astar_max_blocks)),
                   "batch_set_astar_blocks")
            _check(lib().gh_batch_set_knapsack_order(h, KNAPSACK_ORDERS[knapsack_order], int(switch_counter)),
                   "batch_set_knapsack_order")
            for kind, data in instances:
                if kind == "astar":
                    g = np.ascontiguousarray(data, np.uint8)
                    _check(lib().gh_batch_add_astar(h, g.shape[1], g.shape[0], g.ctypes.data, None), "add_astar")
                    self.kinds.append(ASTAR)
                elif kind == "astar8":  # the reference's 8-neighbour bitmap model
                    g = np.ascontiguousarray(data, np.uint8)
                    _check(lib().gh_batch_add_astar_bitmap(h, g.shape[1], g.shape[0], g.ctypes.data, None),
                           "add_astar_bitmap")
                    self.kinds.append(ASTAR)
                else:
                    w, p, cap = data
                    w = np.ascontiguousarray(w, np.int32)
                    p = np.ascontiguousarray(p, np.int32)
                    _check(lib().gh_batch_add_knapsack(h, w.size, w.ctypes.data, p.ctypes.data, int(cap), None),
                           "add_knapsack")
                    self.kinds.append(KNAPSACK)
            _check(lib().gh_batch_build(h, _stream(stream)), "batch_build")
        except Exception:
            self.close()
            raise

    def run(self, mode="graph", stream=None):
        """Starts every search (asynchronous): mode graph / persistent / plain."""
        _check(lib().gh_batch_run(self._h, _MODES[mode], _stream(stream)), "batch_run")

    def results(self, stream=None, check=True):
        """(results int64 per instance, status per instance, stats (count, 3))."""
        n = len(self.kinds)
        res = np.zeros(n, np.int64)
        st = np.zeros(n, np.int32)
        stats = np.zeros((n, 3), np.uint64)
        rc = lib().gh_batch_results(self._h, res.ctypes.data, st.ctypes.data, stats.ctypes.data, _stream(stream))
        if check:
            _check(rc, "batch_results")
        return res, st, stats

    def plain_times(self):
        """Milliseconds of each instance's own launch in the last plain run."""
        out = np.zeros(len(self.kinds), np.float32)
        _check(lib().gh_batch_plain_times(self._h, out.ctypes.data), "batch_plain_times")
        return out

    def knapsack_switches(self, stream=None):
        """Heap/FIFO switches per instance in the last run (knapsack, order "switch")."""
        out = np.zeros(len(self.kinds), np.int32)
        _check(lib().gh_batch_knapsack_switches(self._h, out.ctypes.data, _stream(stream)), "knapsack_switches")
        return out

    def info(self):
        c, t, g, th, ab = _I(), _I(), _I(), _I(), _LL()
        _check(lib().gh_batch_info(self._h, ctypes.byref(c), ctypes.byref(t), ctypes.byref(g), ctypes.byref(th),
                                   ctypes.byref(ab)), "batch_info")
        return {"instances": c.value, "tasks": t.value, "grid": g.value, "block_threads": th.value,
                "arena_bytes": ab.value, "batch_size": self.batch_size, "variant": self.variant}

    def close(self):
        if getattr(self, "_h", None):
            lib().gh_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _stream(s):
    if s is None:
        return None
    return s.cuda_stream if hasattr(s, "cuda_stream") else s


def time_run(batch, mode, reps=3):
    """Median wall seconds of `reps` runs (each synchronized)."""
    import torch
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batch.run(mode)
        batch.results(check=True)
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts))


def _cache_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tune_cache.json")


def autotune(instances, sample=None, seed=7, reps=2, cache=True, log=None, full=True):
    """Picks batch size, node layout (bottom-up / top-down) and A* blocks per
    instance for `instances`.  On a sample (default: two instances per SM,
    so the sample keeps the whole GPU busy as the full set does) it times
    batch size x layout at 2^18 cells per block and at most 8 blocks, then
    the cells per block and the block cap from the best.  With `full`, the
    A* block split -- which decides how the largest grids spread over the
    GPU and so the tail of the whole run -- is then chosen by timing the
    whole set: cells per block in {2^18, 2^19, 2^20} x cap in {4, 8} for the
    best layout, and the runner-up layout at the winning split.  The choice
    is cached per GPU and workload signature."""
    import torch
    if sample is None:
        sample = 2 * torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    sig = {"gpu": torch.cuda.get_device_name(), "count": len(instances), "full": bool(full),
           "astar_cells": int(sum(d.size for k, d in instances if k == "astar")),
           "knap_items": int(sum(len(d[0]) for k, d in instances if k == "knapsack"))}
    key = json.dumps(sig, sort_keys=True)
    path = _cache_path()
    if cache and os.path.exists(path):
        try:
            with open(path) as f:
                got = json.load(f).get(key)
            if got:
                return got
        except Exception:
            pass
    rng = np.random.default_rng(seed)
    idx = sorted(rng.choice(len(instances), size=min(sample, len(instances)), replace=False).tolist())
    sub = [instances[i] for i in idx]
    timings = []

    def trial(cfg, insts=sub, n=reps, tag="sample"):
        b = Batch(insts, **cfg)
        try:
            b.run("graph")
            b.results()
            t = time_run(b, "graph", n)
        finally:
            b.close()
        timings.append(dict(cfg, seconds=t, on=tag))
        if log:
            log(dict(cfg, seconds=round(t, 5), on=tag))
        return t

    layouts = []
    for bs in (64, 128, 256, 512):
        for v in ("bottomup", "topdown"):
            cfg = dict(batch_size=bs, variant=v, astar_cells_per_block=1 << 18, astar_max_blocks=8)
            layouts.append((trial(cfg), cfg))
    layouts.sort(key=lambda x: x[0])
    best = (layouts[0][1], layouts[0][0])
    for c in (1 << 16, 1 << 17, 1 << 19, 1 << 20):
        cfg = dict(best[0], astar_cells_per_block=c)
        t = trial(cfg)
        if t < best[1]:
            best = (cfg, t)
    for mb in (4, 16, 32):
        cfg = dict(best[0], astar_max_blocks=mb)
        t = trial(cfg)
        if t < best[1]:
            best = (cfg, t)
    sample_best = best
    if full and len(sub) < len(instances):
        fbest = None
        for c in (1 << 18, 1 << 19, 1 << 20):
            for mb in (4, 8):
                cfg = dict(best[0], astar_cells_per_block=c, astar_max_blocks=mb)
                t = trial(cfg, instances, 1, "full")
                if fbest is None or t < fbest[1]:
                    fbest = (cfg, t)
        second = layouts[1][1]
        cfg = dict(second, astar_cells_per_block=fbest[0]["astar_cells_per_block"],
                   astar_max_blocks=fbest[0]["astar_max_blocks"])
        t = trial(cfg, instances, 1, "full")
        if t < fbest[1]:
            fbest = (cfg, t)
        best = fbest
    choice = dict(best[0], sample=len(sub), sample_seconds=round(sample_best[1], 5),
                  full_seconds=round(best[1], 5) if best is not sample_best else None)
    if cache:
        try:
            data = {}
            if os.path.exists(path):
                with open(path) as f:
                    data = json.load(f)
            data[key] = choice
            with open(path, "w") as f:
                json.dump(data, f, indent=1)
        except Exception:
            pass
    return choice
