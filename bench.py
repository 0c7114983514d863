#!/usr/bin/env python
"""Plain heap-sort benchmark of the GB300 batched priority queue.

One step = one heap-sort through the library: reset the heap, insert all N
keys in insertion() calls of batch_size keys over the whole grid, then
deleteRoot/deleteUpdate until empty (test/partial_heap_test.cu:88-176 without
its concurrent phase; artifacts/synthetic/sort.cu "insdel").  Metric: M keys/s
insert+delete = N / (t_insert + t_delete) per step, whole job over all ranks.

  value     device-resident keys: the timed region holds K back-to-back steps
  e2e       the same through the C ABI with HOST buffers: every step copies the
            keys in from pinned memory and the sorted keys back out
  roofline  the dominant kernel (insert or delete drivers) against the measured
            HBM copy bandwidth, from the closed-form algorithmic bytes
  cpu_baseline  std::sort on the host cores (the reference tests' own CPU
            oracle, test/heap_test.cu:121) over a bounded sample

The heap path does not shard (one global root): with --gpus N every rank runs
an independent replica and `value` sums the replicas (scaling "weak").

--impl reference times the CPU implementation of the path instead (rank 0
only): the oracle's std::sort of the same keys on all host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "M keys/s insert+delete, 2^{log2n} {key}"
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--log2n", type=int, default=28)
    p.add_argument("--batch", type=int, default=2048)
    p.add_argument("--variant", choices=["bottomup", "topdown"], default="bottomup")
    p.add_argument("--no-partial", action="store_true")
    p.add_argument("--key", choices=["u32", "u64"], default="u32")
    p.add_argument("--dist", choices=["uniform", "sorted", "reverse", "zipf"], default="uniform")
    p.add_argument("--grid", type=int, default=0, help="blocks (0: one per SM)")
    p.add_argument("--owner-depth", type=int, default=-1,
                   help="owner-mode bulk delete: resident depth 2..4, 0 off, -1 automatic")
    p.add_argument("--threads", type=int, default=0, help="threads per block (0: automatic)")
    p.add_argument("--tune", action="store_true",
                   help="heapsort: pick batch size, layout, threads, blocks and owner depth with the autotuner "
                        "(gpuheap_gb300.tune) on a 2^24 sample first")
    p.add_argument("--seed", type=int, default=2026)
    p.add_argument("--cpu-sample-log2", type=int, default=28)
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--timeout", type=float, default=2.0,
                   help="heap-sort and FIFO: device wait limit in seconds (raise it under a profiler)")
    p.add_argument("--search-timeout", type=float, default=20.0,
                   help="SSSP and batched searches: device wait limit in seconds (a search block can idle for as "
                        "long as the largest instance runs)")
    p.add_argument("--workload", choices=["heapsort", "sssp", "batched", "served", "fifo"], default="heapsort",
                   help="heapsort: the plain heap-sort line (default); sssp: SSSP with the queue; "
                        "batched: grid A* + knapsack searches in one persistent launch vs per-instance launches; "
                        "served: Poisson streams of SSSP + A* queries through the continuous-batching server; "
                        "fifo: push then pop 2^log2n keys through the device FIFO buffer")
    p.add_argument("--fifo-chunk", type=int, default=0,
                   help="fifo: keys per insertToBuffer/deleteFromBuffer (0: one reservation per call)")
    p.add_argument("--fifo-piece", type=int, default=1024,
                   help="fifo: piece size of the secondary piece-by-piece measurement (0: skip)")
    p.add_argument("--fifo-threads", type=int, default=512, help="fifo: threads per block")
    p.add_argument("--rates", default="100,500,1000,5000", help="served: arrival rates (req/s)")
    p.add_argument("--queries", type=int, default=600, help="served: queries per rate")
    p.add_argument("--plain-queries", type=int, default=48, help="served: queries run alone for the baseline")
    p.add_argument("--batches-per-step", type=int, default=32, help="served: batches a block takes per query per step")
    p.add_argument("--served-batch", type=int, default=1024, help="served: batch size of every query's heap")
    p.add_argument("--served-mode", choices=["device", "host"], default="device",
                   help="served: the device-resident request loop, or one host step per launch")
    p.add_argument("--idle-ms", type=int, default=100, help="served, device loop: idle limit of its launch")
    p.add_argument("--no-host-steps", action="store_true",
                   help="served, device loop: skip the host-step comparison at the same rates")
    p.add_argument("--instances", type=int, default=1024, help="batched: searches per step")
    p.add_argument("--plain-steps", type=int, default=1, help="batched: timed runs of the per-instance launches")
    p.add_argument("--no-tune", action="store_true", help="batched: skip the autotuner (batch 256, bottom-up)")
    p.add_argument("--knapsack-order", choices=["heap", "fifo", "switch"], default="heap",
                   help="batched: knapsack search order (the reference's heap, FIFO and switch models)")
    p.add_argument("--astar-share", type=float, default=0.5, help="batched: fraction of A* instances")
    p.add_argument("--batched-config", default="",
                   help="batched: fixed batch_size,variant,astar_cells_per_block,astar_max_blocks instead of tuning")
    p.add_argument("--scale", type=int, default=22, help="sssp: R-MAT scale")
    p.add_argument("--sources", type=int, default=32, help="sssp: seeded random sources (one per step)")
    p.add_argument("--cpu-sources", type=int, default=16, help="sssp: sources in the CPU Dijkstra sample")
    p.add_argument("--retrieve-sources", type=int, default=4,
                   help="sssp: sources also run through the retrieving heap (gh_sssp_retrieve); 0 skips it")
    args = p.parse_args()
    if args.workload == "sssp":
        if "--steps" not in sys.argv:
            args.steps = args.sources
    return args


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(ms, dist, device):
    """The slowest rank's time: the timed region ends when every rank's work
    has; `dist` is None for one rank."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([float(ms)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world_size, steps, ms):
    """Whole-job rate in M units/s: every rank's units over the max-over-ranks time."""
    return units_per_rank * world_size * steps / (ms / 1e3) / 1e6


# ------------------------------------------------------------------ byte model
def floor_log2_sum(M):
    """sum_{k=1..M} floor(log2 k)."""
    s, l = 0, 0
    while (1 << l) <= M:
        lo, hi = 1 << l, min(M, (1 << (l + 1)) - 1)
        s += l * (hi - lo + 1)
        l += 1
    return s


def algorithmic_bytes(n, B, s, pb):
    """Closed-form BGPQ node traffic of one heap-sort, split by phase:
    insert = s[n + sum_k 2B(L(k)+1) + pb 2BM], delete = s[n + sum_m B(1+3L(m)) + pb 2BM]."""
    M = (n + B - 1) // B
    SL = floor_log2_sum(M)
    ins = s * (n + 2 * B * (SL + M) + (2 * B * M if pb else 0))
    dele = s * (n + B * (M + 3 * SL) + (2 * B * M if pb else 0))
    return ins, dele


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(kernel, args, pb):
    """DRAM bytes of one `kernel` launch as ncu measured them on this exact
    workload (profiles/traffic.json), or None where no capture was taken.
    Never scaled from another size: node traffic reaching DRAM grows faster
    than the keys, as L2 holds a shrinking share of the upper levels."""
    if args.grid or args.threads:
        return None
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            d = json.load(f)
        e = d[f"{kernel}/{args.variant}/{'pb' if pb else 'np'}/B{args.batch}/{args.key}/{args.dist}/2^{args.log2n}"]
        return e["read"] + e["write"]
    except (OSError, KeyError, ValueError):
        return None


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ CPU legs
def cpu_sort_leg(log2n, seed, threads, reps):
    """std::sort on `threads` host cores over a 2^log2n-key sample; M keys/s."""
    import numpy as np
    from oracle import pyoracle
    n = 1 << log2n
    base = pyoracle.gen("u32", seed, "uniform", n)
    times = []
    for _ in range(reps):
        a = base.copy()
        t0 = time.perf_counter()
        pyoracle.sort(a, threads=threads)
        times.append(time.perf_counter() - t0)
    assert np.all(a[1:] >= a[:-1])
    return n / statistics.median(times) / 1e6, times


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n_sample = min(args.cpu_sample_log2, args.log2n)
    import numpy as np
    from oracle import pyoracle
    n = 1 << n_sample
    base = pyoracle.gen("u32", args.seed, args.dist, n)
    for _ in range(args.warmup):
        a = base.copy()
        pyoracle.sort(a, threads=threads)
    times = []
    for _ in range(args.steps):
        a = base.copy()
        t0 = time.perf_counter()
        pyoracle.sort(a, threads=threads)
        times.append(time.perf_counter() - t0)
    assert np.all(a[1:] >= a[:-1])
    total = sum(times)
    value = n * len(times) / total / 1e6
    sample = (f"std::sort (per-thread std::sort + pairwise std::merge) of 2^{n_sample} u32 {args.dist} keys "
              f"per step on {threads} host threads; the reference has no CPU heap, its tests' CPU oracle is std::sort")
    line = {
        "impl": "reference", "metric": METRIC.format(log2n=args.log2n, key="u32"), "value": round(value, 3), "unit": "M keys/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * total / len(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(args),
        "cpu_baseline": {"value": round(value, 3), "unit": "M keys/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "M keys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args):
    pb = not args.no_partial
    name = {("bottomup", True): "buitdd", ("bottomup", False): "buitdd_np", ("topdown", True): "tditdd",
            ("topdown", False): "tditdd_np"}[(args.variant, pb)]
    return {"workload": f"plain heap-sort, 2^{args.log2n} {args.key} keys ({args.dist}, seeded), "
                        f"batch_size {args.batch}, {name}, HEAP_SORT output",
            "n_keys": 1 << args.log2n, "batch_size": args.batch, "variant": name, "key": args.key,
            "distribution": args.dist, "global_batch": 1 << args.log2n,
            "l2": "inputs and heap larger than L2 (129 MB); no flush needed",
            "parallelism": f"replicas x{args.gpus}"}


def owner_summary(st, sm_mhz):
    """Per-delete breakdown of the owner-mode bulk delete of the last step
    (device SM-cycle counters / the SM clock sampled during the run)."""
    d = st.get("deletes", 0)
    if not d:
        return None
    mhz = sm_mhz or 2070.0
    us = lambda k: round(st[k] / d / mhz, 3)
    return {"deletes": d, "lends": st["lends"], "reloads": st["reloads"], "general_steps": st["general_steps"],
            "us_per_delete": {k: us(k) for k in ("loop", "wait_carried", "wait_lent", "wait_ring", "plan", "plan_read",
                                                 "pass", "pass_work", "pass_sync")},
            "taker_us_per_delete": {k: us(k) for k in ("take_lock", "take_load", "take_idle")}}


# ------------------------------------------------------------------ our arm
def our_arm(args):
    import torch

    import gpuheap_gb300 as gh

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    n = 1 << args.log2n
    pb = not args.no_partial
    tuned = None
    if args.tune:
        # the plain path's autotuner on a 2^min(24, log2n) sample of this workload
        from gpuheap_gb300 import tune
        tuned = tune.autotune_sort(log2n=min(24, args.log2n), key=args.key, dist=args.dist, partial_buffer=pb)
        args.batch, args.variant = tuned["batch_size"], tuned["variant"]
        args.threads, args.grid, args.owner_depth = tuned["threads"], tuned["grid"], tuned["owner_depth"]
    B = args.batch
    s = 8 if args.key == "u64" else 4
    tdt = torch.int64 if args.key == "u64" else torch.int32
    bn = 1
    while bn * B < 2 * n:
        bn <<= 1

    stream = torch.cuda.Stream()
    keys = gh.gen_keys(args.key, args.seed + rank, args.dist, n)
    want = gh.sort_keys(keys, args.key)  # the property the output must meet, by torch
    out = torch.empty_like(keys)
    h = gh.Heap(bn, B, key=args.key, variant=args.variant, partial_buffer=pb)
    if args.grid:
        h.set_grid(args.grid)
    if args.threads:
        h.set_block_threads(args.threads)
    if args.owner_depth != -1:
        h.set_owner_depth(args.owner_depth)
    h.set_timeout(args.timeout)
    info = h.info()
    torch.cuda.synchronize()

    def step(ev=None):
        with torch.cuda.stream(stream):
            if ev:
                ev[0].record(stream)
            h.reset_async(stream)
            if ev:
                ev[1].record(stream)
            h.insert(keys, chunk=B, stream=stream)
            if ev:
                ev[2].record(stream)
            h.delete(out, stream=stream, sync=False)
            if ev:
                ev[3].record(stream)

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    h.sync(stream)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = gh.launch_count()
    barrier()
    with ClockSampler(local) as clk:
        start.record(stream)
        for k in range(args.steps):
            step(evs[k])
        end.record(stream)
        stream.synchronize()
    barrier()
    launches = gh.launch_count() - launches0
    h.sync(stream)
    total_ms = start.elapsed_time(end)
    t_reset = [e[0].elapsed_time(e[1]) for e in evs]
    t_ins = [e[1].elapsed_time(e[2]) for e in evs]
    t_del = [e[2].elapsed_time(e[3]) for e in evs]
    total_ms = max_over_ranks(total_ms, dist, "cuda")

    # the owner's counters of the last timed step's bulk delete (the e2e
    # steps below delete in pieces and would leave a piece's counters)
    owner = owner_summary(h.owner_stats(), clk.summary().get("sm_mhz"))

    # correctness of the last step: the deleted stream is the input in key order
    if not torch.equal(out, want):
        raise SystemExit("bench: heap-sort output is not the input in key order")

    # e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        host_in = keys.cpu().pin_memory()
        host_out = torch.empty(n, dtype=tdt).pin_memory()

        def e2e_step():
            # the C ABI's host-buffer heap-sort: copies in pieces on the
            # heap's own stream, overlapped with the inserts and deletes
            h.sort_host(host_in, host_out, stream=stream)

        for _ in range(max(1, min(args.warmup, 2))):
            e2e_step()
        stream.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e1.record(stream)
        stream.synchronize()
        e2e_ms = e0.elapsed_time(e1)
        e2e_ms = max_over_ranks(e2e_ms, dist, "cuda")
        if not torch.equal(host_out, want.cpu()):
            raise SystemExit("bench: e2e output is not the input in key order")
        e2e = {"value": round(job_rate(n, ws, args.steps, e2e_ms), 3), "unit": "M keys/s",
               "h2d_bytes_per_step": n * s, "d2h_bytes_per_step": n * s,
               "ms_per_step": round(e2e_ms / args.steps, 3),
               "path": "pinned host keys -> gh_heap_sort_host (8 pieces each way, copies overlapped with the "
                       "inserts and deletes) -> pinned host output"}

    value = job_rate(n, ws, args.steps, total_ms)
    ins_b, del_b = algorithmic_bytes(n, B, s, pb)
    ti, td = statistics.mean(t_ins), statistics.mean(t_del)
    del_kern = "k_delete_owner" if owner else "k_delete"  # the owner launch does all but the last few deletes
    ins_kern = "k_insert_reserved"  # full batches (chunk = batch_size) into reserved targets
    kern, kb, kt = (del_kern, del_b, td) if td >= ti else (ins_kern, ins_b, ti)
    peak, peak_kind = peaks()
    achieved = kb / (kt / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 5), "traffic": ncu_traffic(kern, args, pb),
            "kernel": kern, "peak_source": f"{peak_kind} hbm_gbs",
            "algorithmic_bytes": kb, "launch_ms": round(kt, 3),
            "note": "achieved = closed-form BGPQ node bytes of the phase / its CUDA-event time (for deletes: the "
                    "owner-mode launch plus the plain k_delete for the last few nodes); frac of measured; traffic = ncu "
                    "DRAM read+write bytes of one launch of this kernel on this workload (1 pass), null if not captured"}
    line = {
        "metric": METRIC.format(log2n=args.log2n, key=args.key), "value": round(value, 3), "unit": "M keys/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.key, "data": "synthetic",
        "config": dict(workload_config(args), block_threads=info["block_threads"], grid=info["grid"],
                       **({"tuned": tuned} if tuned else {})),
        "phases_ms": {"reset": round(statistics.mean(t_reset), 3), "insert": round(ti, 3), "delete": round(td, 3)},
        "roofline": roof, "e2e": e2e, "gpu_launches": launches, "clocks": clk.summary(),
        "owner_delete": owner,
        "whole_sort_bytes_per_key": round((ins_b + del_b) / n, 2),
        "io_lower_bound_bytes_per_key": 2 * s,
    }
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, times = cpu_sort_leg(min(args.cpu_sample_log2, args.log2n), args.seed, threads, reps=3)
        line["cpu_baseline"] = {"value": round(v, 3), "unit": "M keys/s", "cores": threads, "kind": "port",
                                "sample": f"std::sort of 2^{min(args.cpu_sample_log2, args.log2n)} u32 uniform keys "
                                          f"on {threads} threads (per-thread std::sort + pairwise std::merge), "
                                          f"median of 3"}
        log2s = min(24, args.log2n)
        v1, _ = cpu_sort_leg(log2s, args.seed, 1, reps=1)
        line["cpu_single_thread"] = {"value": round(v1, 3), "unit": "M keys/s", "cores": 1,
                                     "sample": f"std::sort of 2^{log2s} u32 uniform keys on one thread, once"}
    h.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ------------------------------------------------------------------ SSSP
SSSP_METRIC = "SSSP ms per source, R-MAT scale {scale} (edge factor 16, weights 1-1000), u64 dist<<32|v keys"


def sssp_sources(rowptr, k, seed):
    import numpy as np
    deg = np.diff(rowptr)
    return np.random.default_rng(seed).choice(np.nonzero(deg)[0], size=k, replace=False)


def sssp_cpu_leg(host, sources, threads):
    """CPU Dijkstra (std::priority_queue) of the sample sources: the oracle
    distances and the single-thread and all-core times."""
    from oracle import pyoracle
    t0 = time.perf_counter()
    one = pyoracle.dijkstra(*host, sources[:1], threads=1)
    t1 = time.perf_counter() - t0
    t0 = time.perf_counter()
    alld = pyoracle.dijkstra(*host, sources, threads=threads)
    tall = time.perf_counter() - t0
    return alld, one, t1, tall


def sssp_arm(args):
    """One step = single-source shortest paths from one seeded source through
    gh_sssp (the heap-driven label-correcting kernel); the timed region holds
    `steps` sources back to back with the graph resident in HBM."""
    import numpy as np
    import torch

    import gpuheap_gb300 as gh
    from gpuheap_gb300 import sssp as gs

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    g = gs.rmat_graph(args.scale, 16, seed=args.seed)
    torch.cuda.synchronize()
    host = g.host()
    srcs = sssp_sources(host[0], max(args.sources, args.steps), args.seed)
    heap = gs.make_heap(g, batch_size=args.batch, variant=args.variant)
    if args.grid:
        heap.set_grid(args.grid)
    heap.set_timeout(args.search_timeout)
    info = heap.info()
    for i in range(args.warmup):
        gs.sssp(heap, g, int(srcs[i % len(srcs)]))
    l0 = gh.launch_count()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    per, keys, edges, dists = [], 0, 0, []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev[0].record()
        for i in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dist, st = gs.sssp(heap, g, int(srcs[i]))
            e1.record()
            e1.synchronize()
            per.append(e0.elapsed_time(e1))
            keys += st["keys_taken"]
            edges += st["edges_scanned"]
            if i < args.cpu_sources:
                dists.append(dist.cpu().numpy().view(np.uint32).copy())
        ev[1].record()
        torch.cuda.synchronize()
    total_ms = ev[0].elapsed_time(ev[1])
    launches = gh.launch_count() - l0
    per_sorted = sorted(per)
    value = statistics.mean(per)
    line = {
        "metric": SSSP_METRIC.format(scale=args.scale), "value": round(value, 2), "unit": "ms/source",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 2),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"SSSP from {args.steps} seeded sources, R-MAT scale {args.scale}, edge factor 16, "
                               f"a=0.57 b=0.19 c=0.19, symmetrised, u32 weights 1-1000; "
                               f"batch_size {args.batch} {args.variant} with partial buffer",
                   "vertices": g.n, "directed_edges": g.m, "batch_size": args.batch, "variant": args.variant,
                   "block_threads": info["block_threads"], "grid": info["grid"],
                   "l2": "graph (CSR) and distances larger than L2", "parallelism": f"replicas x{ws}"},
        "p50_ms": round(per_sorted[len(per) // 2], 2), "p99_ms": round(per_sorted[min(len(per) - 1, int(0.99 * len(per)))], 2),
        "edges_per_s": round(g.m * args.steps / (total_ms / 1e3), 1),
        "scanned_edges_per_source": round(edges / args.steps), "keys_taken_per_source": round(keys / args.steps),
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    # the reference application's own form: the retrieving heap with the
    # auxiliary buffer (gh_sssp_retrieve), at the reference's configuration
    # (batch 512, 256-edge chunks, 10 blocks: sssp_config.cuh) and at batch
    # 1024 with 64-edge chunks on 24 blocks; each call allocates its heap
    if args.retrieve_sources > 0:
        forms = {}
        k = min(args.retrieve_sources, args.steps)
        for name, (bsz, chunk, blocks) in (("reference_config", (512, 256, 10)), ("b1024_c64_x24", (1024, 64, 24))):
            gs.sssp_retrieve(g, int(srcs[0]), batch_size=bsz, chunk=chunk, blocks=blocks)  # warm-up
            times, same = [], True
            for i in range(k):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                d2, st2 = gs.sssp_retrieve(g, int(srcs[i]), batch_size=bsz, chunk=chunk, blocks=blocks)
                e1.record()
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
                if i < len(dists):
                    same = same and bool(np.array_equal(d2.cpu().numpy().view(np.uint32), dists[i]))
            if not same:
                raise SystemExit("bench: SSSP through the retrieving heap differs from gh_sssp")
            forms[name] = {"batch_size": bsz, "chunk": chunk, "blocks": blocks,
                           "ms_per_source": round(statistics.mean(times), 2),
                           "handovers_last_source": st2["handovers"]}
        line["retrieving_heap_form"] = dict(forms, sources=k, note="gh_sssp_retrieve (the reference's ssspKernel "
                                            "on its retrieving heap with the auxiliary buffer); distances equal "
                                            "gh_sssp's; each call allocates its heap")
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        k = min(args.cpu_sources, args.steps)
        want, _, t1, tall = sssp_cpu_leg(host, srcs[:k], threads)
        exact = all(np.array_equal(dists[i], want[i]) for i in range(k))
        if not exact:
            raise SystemExit("bench: SSSP distances differ from CPU Dijkstra")
        line["exact_vs_dijkstra"] = f"{k} of {k} sources bit-exact"
        line["cpu_baseline"] = {"value": round(1e3 * t1, 2), "unit": "ms/source", "cores": 1, "kind": "port",
                                "sample": f"std::priority_queue Dijkstra of 1 source on 1 thread; all {threads} "
                                          f"cores, one source per thread: {round(1e3 * tall / k, 2)} ms/source "
                                          f"over {k} sources"}
    heap.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ batched searches
BATCHED_METRIC = "searches/s, {count} grid A* + knapsack instances per launch"


def batched_cpu_leg(inst, threads):
    """The oracle on every instance, one instance per task on `threads` cores."""
    import numpy as np
    from oracle import pyoracle
    t0 = time.perf_counter()
    grids = [d for k, d in inst if k == "astar"]
    knaps = [d for k, d in inst if k == "knapsack"]
    a = iter(pyoracle.astar_grid_many(grids, threads=threads))
    k = iter(pyoracle.knap_bb_many(knaps, threads=threads))
    want = np.array([int(next(a)) if kind == "astar" else int(next(k)) for kind, _ in inst], np.int64)
    return want, time.perf_counter() - t0


def batched_arm(args):
    """One step = every search of the workload once, from scratch, as one
    graph-replayed persistent launch (fill + seed + search + collect)."""
    import numpy as np
    import torch

    import gpuheap_gb300 as gh
    from gpuheap_gb300 import batch as gb

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    inst = gb.workload(count=args.instances, seed=args.seed, astar_share=args.astar_share)
    gen_s = time.perf_counter() - t0
    if args.batched_config:
        bs, var, cells, mb = args.batched_config.split(",")
        cfg = {"batch_size": int(bs), "variant": var, "astar_cells_per_block": int(cells),
               "astar_max_blocks": int(mb), "fixed": True}
    elif args.no_tune:
        cfg = {"batch_size": 256, "variant": "bottomup", "astar_cells_per_block": 1 << 18, "astar_max_blocks": 8}
    else:
        cfg = gb.autotune(inst)
    b = gb.Batch(inst, batch_size=cfg["batch_size"], variant=cfg["variant"],
                 astar_cells_per_block=cfg["astar_cells_per_block"], astar_max_blocks=cfg.get("astar_max_blocks", 8),
                 timeout=args.search_timeout, knapsack_order=args.knapsack_order)
    info = b.info()
    stream = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 1)):
        b.run("graph", stream)
    b.results(stream, check=args.knapsack_order == "heap")
    l0 = gh.launch_count()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev[0].record(stream)
        for _ in range(args.steps):
            b.run("graph", stream)
        ev[1].record(stream)
        torch.cuda.synchronize()
    batched_ms = ev[0].elapsed_time(ev[1]) / args.steps
    launches = gh.launch_count() - l0
    res, st, stats = b.results(stream, check=args.knapsack_order == "heap")
    failed = np.nonzero(st)[0]
    # the baseline: one launch per instance, each instance with the best of
    # three setups (the batched tuning; a lone A* grid on up to 64 blocks of
    # 2^16 cells; up to 16 blocks of 2^18 cells), timed per launch
    plain_ms, plain_identical, plain_setups = None, None, {}
    if args.plain_steps > 0:
        setups = [("batched tuning", cfg),
                  ("wide", dict(cfg, astar_cells_per_block=1 << 16, astar_max_blocks=64)),
                  ("middle", dict(cfg, astar_cells_per_block=1 << 18, astar_max_blocks=16))]
        best, plain_identical = None, True
        for name, c in setups:
            pb = b if name == "batched tuning" else gb.Batch(
                inst, batch_size=c["batch_size"], variant=c["variant"],
                astar_cells_per_block=c["astar_cells_per_block"], astar_max_blocks=c["astar_max_blocks"],
                timeout=args.search_timeout, knapsack_order=args.knapsack_order)
            runs = []
            for _ in range(args.plain_steps):
                pb.run("plain", stream)
                runs.append(pb.plain_times())
            per = np.mean(np.stack(runs), axis=0)
            r, s_, _ = pb.results(stream)
            plain_identical = plain_identical and bool(np.array_equal(r, res) and not s_.any())
            plain_setups[name] = round(float(per.sum()), 1)
            best = per if best is None else np.minimum(best, per)
            if pb is not b:
                pb.close()
        plain_ms = float(best.sum())
    kinds = np.array([0 if k == "astar" else 1 for k, _ in inst])
    count = len(inst)
    line = {
        "metric": BATCHED_METRIC.format(count=count), "value": round(count / (batched_ms / 1e3), 2),
        "unit": "searches/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(batched_ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"{int((kinds == 0).sum())} grid A* (side log-uniform 256-4096, 20% obstacles, "
                               f"costs 1-9, Manhattan heuristic) + {int((kinds == 1).sum())} 0/1 knapsack "
                               f"(100-1000 items, weights 1-1000, profit = weight + U(0,100), capacity half "
                               f"the weight), seed {args.seed}",
                   "tuned": cfg, "knapsack_order": args.knapsack_order,
                   "grid": info["grid"], "tasks": info["tasks"], "block_threads": info["block_threads"],
                   "arena_bytes": info["arena_bytes"], "generate_s": round(gen_s, 2),
                   "l2": "grids and distance arrays larger than L2; every step resets them",
                   "parallelism": f"replicas x{ws}"},
        "plain_ms_per_step": round(plain_ms, 3) if plain_ms else None,
        "plain_setups_ms": plain_setups or None,
        "plain_note": "one launch per instance, each instance timed alone (events around its launch) in three "
                      "setups; plain_ms_per_step sums every instance's best",
        "batched_vs_plain": round(plain_ms / batched_ms, 2) if plain_ms else None,
        "plain_results_identical": plain_identical,
        "expansions_per_s": round(float(stats[:, 1].sum()) / (batched_ms / 1e3), 1),
        "keys_taken_per_step": int(stats[:, 0].sum()), "keys_inserted_per_step": int(stats[:, 2].sum()),
        "failed_instances": int(len(failed)),
        "knapsack_switches": int(b.knapsack_switches(stream).sum()),
        "astar_cells": int(sum(d.size for k, d in inst if k == "astar")),
        "gpu_launches_per_step": round(launches / args.steps, 2),
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        want, cpu_s = batched_cpu_leg(inst, threads)
        ok = np.ones(count, bool)
        ok[failed] = False  # an instance that ran out of its pool or ring reports GH_ERR_CAPACITY
        if not np.array_equal(res[ok], want[ok]):
            bad = np.nonzero((res != want) & ok)[0]
            raise SystemExit(f"bench: batched results differ from the CPU oracle at instances {bad[:10].tolist()}")
        line["exact_vs_cpu"] = (f"{int(ok.sum())} of {count} instances equal the CPU A* / branch-and-bound optimum"
                                + (f"; {len(failed)} reported GH_ERR_CAPACITY" if len(failed) else ""))
        line["cpu_baseline"] = {"value": round(count / cpu_s, 2), "unit": "searches/s", "cores": threads,
                                "kind": "port", "sample": f"all {count} instances, one per task on {threads} "
                                                          f"threads (std::priority_queue A*, best-first B&B)"}
    b.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ served queries
SERVED_METRIC = "served queries/s at {rate} req/s offered, mixed SSSP (R-MAT 16-22) + grid A* (256^2-4096^2)"
SSSP_SCALES = (16, 18, 20, 22)
MAP_SIDES = (256, 512, 1024, 2048, 4096)


def served_queries(graphs, maps, count, seed):
    """Half SSSP, half A*; within each, size class k (0 = smallest) has weight
    4^-k, so every class brings about the same work."""
    import numpy as np
    from gpuheap_gb300 import serve as gs
    rng = np.random.default_rng(seed)
    ws = np.array([4.0 ** -k for k in range(len(graphs))]); ws /= ws.sum()
    wm = np.array([4.0 ** -k for k in range(len(maps))]); wm /= wm.sum()
    out = []
    for _ in range(count):
        if rng.random() < 0.5:
            gi = int(rng.choice(len(graphs), p=ws))
            out.append((gs.SSSP, gi, int(rng.integers(graphs[gi].n)), 0))
        else:
            mi = int(rng.choice(len(maps), p=wm))
            cells = maps[mi].numel()
            out.append((gs.ASTAR, len(graphs) + mi, int(rng.integers(cells)), int(rng.integers(cells))))
    return out


def served_cpu_leg(graphs_host, maps_host, queries, threads):
    """Oracle results (SSSP digest, A* cost) of `queries` and the CPU time
    per query: Dijkstra / A* one query per thread."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    from oracle import pyoracle
    ng = len(graphs_host)

    def one(q):
        k, d, a, b = q
        if k == 2:
            dist = pyoracle.dijkstra(*graphs_host[d], [a])[0]
            fin = dist != 0xFFFFFFFF
            return int(fin.sum()), int(dist[fin].astype(np.uint64).sum())
        return int(pyoracle.astar_grid_sg(maps_host[d - ng], a, b)), 0

    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(one, queries))
    return res, time.perf_counter() - t0


def served_arm(args):
    """Per offered rate: `queries` seeded queries arrive by a Poisson process
    and go through the server -- by default its device-resident request loop
    (admission by free memory, setup, search, collection and freeing inside
    one persistent launch; the host posts requests and reads completions),
    then, for comparison, its host steps (one launch and one synchronization
    per step); latency = completion seen by the host - arrival.  The
    baseline runs a sample of the same mix one query at a time, each alone
    on the GPU, in one launch, until it finishes."""
    import numpy as np
    import torch

    import gpuheap_gb300 as gh
    from gpuheap_gb300 import batch as gb
    from gpuheap_gb300 import serve as gs
    from gpuheap_gb300 import sssp as gsssp

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    graphs = [gsssp.rmat_graph(s, 16, seed=args.seed + s) for s in SSSP_SCALES]
    maps_host = [gb.gen_grid(side, args.seed + side) for side in MAP_SIDES]
    maps = [torch.from_numpy(m).cuda() for m in maps_host]
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0

    def server(**kw):
        s = gs.Server(**kw)
        for g in graphs:
            s.add_graph(g)
        for m in maps:
            s.add_map(m)
        return s

    rates = [float(r) for r in args.rates.split(",")]
    device_loop = args.served_mode == "device"

    def serve_rates(resident):
        """Every offered rate through one server: the device-resident loop
        (resident) or host steps.  Returns (per-rate records, launches)."""
        srv = server(max_slots=256, batch_size=args.served_batch, batches_per_step=args.batches_per_step)
        if resident:
            srv.start(idle_ms=args.idle_ms)
        warm = served_queries(graphs, maps, 8, args.seed + 99)
        gs.run_stream(srv, warm, np.zeros(len(warm)), resident=resident)
        if resident:  # the loop's launch leaves; the first poll of the timed streams launches it again
            srv.stop()
            srv.start(idle_ms=args.idle_ms)
        out, l0 = [], gh.launch_count()
        for i, rate in enumerate(rates):
            qs = served_queries(graphs, maps, args.queries, args.seed + i)
            arr = gs.poisson_arrivals(len(qs), rate, args.seed + 1000 + i)
            lat, res, makespan, steps = gs.run_stream(srv, qs, arr, resident=resident)
            bad = [r for r in res if r[0] != gs.FINISHED]
            if bad:
                raise SystemExit(f"bench: {len(bad)} served queries failed at {rate} req/s")
            out.append({"offered_per_s": rate, "queries": len(qs), "served_per_s": round(len(qs) / makespan, 2),
                        "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
                        "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 2),
                        "makespan_s": round(makespan, 3), ("polls" if resident else "steps"): steps})
        launches = gh.launch_count() - l0
        if resident:
            out[-1]["loop_launches"] = srv.info()["steps"]
        srv.close()
        return out, launches

    with ClockSampler(local) as clk:
        per_rate, launches = serve_rates(device_loop)
    host_rates = serve_rates(False)[0] if device_loop and not args.no_host_steps else None
    # baseline: a sample of the same mix, one query at a time, each alone on the
    # GPU in the configuration that suits it best: SSSP through the standalone
    # kernel (gh_sssp, batch 2048 on 24 blocks), A* alone in the engine
    plain_q = served_queries(graphs, maps, args.plain_queries, args.seed + 777)
    sssp_heaps = {}
    alone = server(max_slots=1, batch_size=args.served_batch, batches_per_step=1 << 20)
    secs, res_alone = [], []
    for k, d, a, b2 in plain_q:
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        if k == gs.SSSP:
            if d not in sssp_heaps:
                sssp_heaps[d] = gsssp.make_heap(graphs[d])
                t1 = time.perf_counter()
            dist, _ = gsssp.sssp(sssp_heaps[d], graphs[d], a)
            torch.cuda.synchronize()
            secs.append(time.perf_counter() - t1)
            dv = dist.to(torch.int64) & 0xFFFFFFFF  # u32 distances held in int32
            fin = dv != 0xFFFFFFFF
            res_alone.append((gs.FINISHED, int(fin.sum().item()), int(dv[fin].sum().item()), 0))
        else:
            q = alone.submit(k, d, a, b2)
            while q not in alone.step()[0]:
                pass
            secs.append(time.perf_counter() - t1)
            res_alone.append(alone.result(q))
    alone.close()
    for h in sssp_heaps.values():
        h.close()
    secs = np.array(secs)
    plain_qps = len(plain_q) / float(secs.sum())
    mix = served_queries(graphs, maps, args.plain_queries, args.seed + 777)
    srv = server(max_slots=256, batch_size=args.served_batch, batches_per_step=args.batches_per_step)
    if device_loop:
        srv.start(idle_ms=args.idle_ms)
    _, res_mix, _, _ = gs.run_stream(srv, mix, np.zeros(len(mix)), resident=device_loop)
    srv.close()
    same = [(r[1], r[2]) for r in res_alone] == [(r[1], r[2]) for r in res_mix]
    top = per_rate[-1]
    line = {
        "metric": SERVED_METRIC.format(rate=int(top["offered_per_s"])), "value": top["served_per_s"],
        "unit": "queries/s", "n_gpus": ws, "steps": len(rates), "warmup": 1,
        "ms_per_step": round(1e3 * top["makespan_s"], 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"{args.queries} queries per rate: half SSSP on R-MAT scales {list(SSSP_SCALES)} "
                               f"(edge factor 16, weights 1-1000), half A* on {list(MAP_SIDES)}-side grids "
                               f"(20% obstacles, costs 1-9) between random cells; size class k weighted 4^-k",
                   "batch_size": args.served_batch, "variant": "bottomup", "max_slots": 256,
                   "batches_per_step": args.batches_per_step, "setup_s": round(setup_s, 2),
                   "loop": ("device-resident request loop (pinned request / completion rings, one persistent "
                            f"launch, idle exit after {args.idle_ms} ms)") if device_loop
                           else "host steps (one launch and one synchronization per step)",
                   "parallelism": f"replicas x{ws}"},
        "rates": per_rate, "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
        "plain_per_s": round(plain_qps, 2), "served_vs_plain": round(top["served_per_s"] / plain_qps, 2),
        "alone_equals_mix": f"{len(plain_q)} queries: {'identical' if same else 'DIFFERENT'} results alone and in the mix",
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    if host_rates is not None:
        line["host_step_rates"] = host_rates
    if not same:
        raise SystemExit("bench: served results differ between alone and in the mix")
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sample = plain_q[:threads]
        want, cpu_s = served_cpu_leg([g.host() for g in graphs], maps_host, sample, threads)
        got = [(r[1], r[2]) for r in res_alone[:len(sample)]]
        if got != want:
            raise SystemExit("bench: served results differ from the CPU oracle")
        line["exact_vs_cpu"] = f"{len(sample)} sampled queries equal CPU Dijkstra digests / A* costs"
        line["cpu_baseline"] = {"value": round(len(sample) / cpu_s, 2), "unit": "queries/s", "cores": threads,
                                "kind": "port", "sample": f"{len(sample)} queries of the mix, one per thread "
                                                          f"(std::priority_queue Dijkstra / A*)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ FIFO buffer
FIFO_METRIC = "M keys/s push+pop, 2^{log2n} {key} through the device FIFO buffer"


def fifo_cpu_leg(log2n, chunk, reps):
    """The oracle's sequential Buffer<K> model (numpy ring copies), one thread."""
    import numpy as np
    from oracle import pyoracle
    n = 1 << log2n
    keys = pyoracle.gen("u32", 7, "uniform", n)
    times = []
    for _ in range(reps):
        m = pyoracle.FifoModel(n, np.uint32)
        t0 = time.perf_counter()
        m.push(keys, chunk)
        got = m.pop(n, chunk)
        times.append(time.perf_counter() - t0)
    assert np.array_equal(got, keys)
    return n / statistics.median(times) / 1e6


def fifo_arm(args):
    """One step = push 2^log2n device-resident keys into an empty ring of that
    capacity over the whole grid (insertKernel, bufferTest.cu:39-47), then pop
    them all (deleteKernel, bufferTest.cu:49-56); `chunk` keys per call."""
    import torch

    import gpuheap_gb300 as gh
    from gpuheap_gb300.fifo import Fifo

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    n = 1 << args.log2n
    kb = 8 if args.key == "u64" else 4
    chunk = args.fifo_chunk
    keys = gh.gen_keys(args.key, args.seed, "uniform", n)
    out = torch.empty_like(keys)
    f = Fifo(n, args.key)
    f.set_timeout(args.timeout)
    f.set_launch(threads=args.fifo_threads)
    info = f.info()

    def step(ev=None):
        if ev:
            ev[0].record()
        f.push(keys, chunk=chunk)
        if ev:
            ev[1].record()
        got = f.pop(out, chunk=chunk, sync=ev is None)
        if ev:
            ev[2].record()
        return got

    for _ in range(max(1, args.warmup)):
        assert step() == n
    l0 = gh.launch_count()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            step(evs[i])
            f.count()  # synchronises; the next push then needs no host-side wait
        torch.cuda.synchronize()
    launches = gh.launch_count() - l0
    t_push = [e[0].elapsed_time(e[1]) for e in evs]
    t_pop = [e[1].elapsed_time(e[2]) for e in evs]
    total_ms = sum(t_push) + sum(t_pop)
    value = n * args.steps / (total_ms / 1e3) / 1e6
    # pieces from different blocks may interleave: the output must be a
    # permutation of the input (same multiset, compared sorted on the device)
    if not torch.equal(torch.sort(out).values, torch.sort(keys).values):
        raise SystemExit("bench: FIFO output is not a permutation of its input")

    peak, peak_kind = peaks()
    push_ms, pop_ms = statistics.mean(t_push), statistics.mean(t_pop)
    dom, dom_ms = ("k_fifo_pop", pop_ms) if pop_ms >= push_ms else ("k_fifo_push", push_ms)
    algo = 2 * kb * n  # push: read the input + write the ring; pop: read the ring + write the output
    achieved = algo / (dom_ms / 1e3) / 1e9
    line = {
        "metric": FIFO_METRIC.format(log2n=args.log2n, key=args.key), "value": round(value, 1), "unit": "M keys/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.key, "data": "synthetic",
        "config": {"workload": f"device FIFO: push 2^{args.log2n} {args.key} keys then pop them, ring of 2^{args.log2n}, "
                               + (f"{chunk} keys per call" if chunk else "one reservation per call"), "n_keys": n, "chunk": chunk, "blocks": info["blocks"],
                   "threads": info["threads"], "l2": "keys and ring larger than L2 (129 MB); no flush needed",
                   "parallelism": f"replicas x{ws}"},
        "push_ms": round(push_ms, 3), "pop_ms": round(pop_ms, 3),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": None,
                     "algorithmic_bytes_per_launch": algo},
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    if args.fifo_piece and chunk == 0:
        # the reference's call shape: one insertToBuffer / deleteFromBuffer per piece
        f.push(keys, chunk=args.fifo_piece)
        f.pop(out, chunk=args.fifo_piece)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        f.push(keys, chunk=args.fifo_piece)
        e[1].record()
        assert f.pop(out, chunk=args.fifo_piece) == n
        e[2].record()
        torch.cuda.synchronize()
        ms = e[0].elapsed_time(e[2])
        line["per_piece"] = {"piece": args.fifo_piece, "value": round(n / (ms / 1e3) / 1e6, 1), "unit": "M keys/s",
                             "push_ms": round(e[0].elapsed_time(e[1]), 3), "pop_ms": round(e[1].elapsed_time(e[2]), 3),
                             "note": "pieces publish in reservation order; one hand-off per piece bounds the rate"}
    if not args.no_e2e:
        pinned_in = keys.cpu().pin_memory()
        pinned_out = torch.empty_like(pinned_in).pin_memory()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            keys.copy_(pinned_in, non_blocking=True)
            f.push(keys, chunk=chunk)
            assert f.pop(out, chunk=chunk) == n
            pinned_out.copy_(out, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        line["e2e"] = {"value": round(n * args.steps / (ms / 1e3) / 1e6, 1), "unit": "M keys/s",
                       "h2d_bytes_per_step": n * kb, "d2h_bytes_per_step": n * kb}
    if rank == 0 and not args.no_cpu:
        log2s = min(args.log2n, 26)
        v = fifo_cpu_leg(log2s, chunk or 65536, 3)
        line["cpu_baseline"] = {"value": round(v, 1), "unit": "M keys/s", "cores": 1, "kind": "port",
                                "sample": f"the oracle's sequential Buffer model (numpy ring copies), push then pop "
                                          f"of 2^{log2s} u32 keys in pieces of {chunk or 65536}, 1 thread"}
    f.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "sssp":
        return sssp_arm(args)
    if args.workload == "batched":
        return batched_arm(args)
    if args.workload == "served":
        return served_arm(args)
    if args.workload == "fifo":
        return fifo_arm(args)
    return our_arm(args)


if __name__ == "__main__":
    sys.exit(main())
