"""Generate tests/golden/bgpq_ref_cases.npz from the reference's own heap code.

Runs the reference's Heap<K> (heap/{tditdd,tditdd_np,buitdd,buitdd_np}/heap.cuh,
compiled for the host by oracle/Makefile's `ref` target through
oracle/ref_shim.h, one thread per "block") over seeded operation sequences and
records, per case: the input keys, the operation list, every deleteRoot size,
the HEAP_SORT output buffer, the heap memory and counters after the insert
phase and at the end.  These vectors pin both the oracle restatement (CPU
tests) and the CUDA path (GPU tests, one thread block, where the heap is
deterministic).

Four sets: `small` (bgpq_ref_cases.npz, batch 16-64, every key type and
scenario), `large` (bgpq_ref_cases_large.npz, batch 256-2048, the batch
sizes of the heap-sort configurations), `astar` (astar_ref_cases.npz:
bitmaps through the reference's sequential A*, artifacts/astar/
seq_astar.hpp, pinning the oracle's A* machinery) and `retrieve`
(retrieve_ref_cases.npz: insert / retrieve sequences through the reference's
retrieving heap, applications/sssp_longfei_new/heap.cuh, pinning the runs
that `retrieve` returns and the heap each sequence leaves).

Usage (needs the reference tree; not run by the tests):
    make -C oracle ref REF=<reference tree> && python tests/golden/make_golden.py [small] [large] [retrieve] [astar]
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(REPO, "oracle", "_ref", "libbgpq_ref.so")

TYPES = {
    "u32": (np.uint32, ctypes.c_uint32, 0xFFFFFFFF),
    "u64": (np.uint64, ctypes.c_uint64, 2**64 - 1),
    "i32": (np.int32, ctypes.c_int32, 2**31 - 1),
}
VARIANTS = ["tditdd", "tditdd_np", "buitdd", "buitdd_np"]
VP = ctypes.c_void_p


def keys_for(rng, kind, n, split, ties=False):
    """Seeded keys; with split=True the first half lies below the second half
    (the shape of test/partial_heap_test.cu:114-119); with ties=True they come
    from about 40 values, so equal keys meet in every comparison."""
    dt = TYPES[kind][0]
    if kind == "u64":
        lo, hi = 0, 2**63
    elif kind == "i32":
        lo, hi = -(2**31), 2**31 - 1
    else:
        lo, hi = 0, 2**32 - 1
    if ties:
        return rng.integers(lo, lo + 40, n, dtype=dt)
    if not split:
        return rng.integers(lo, hi, n, dtype=dt)
    mid = lo + (hi - lo) // 2
    a = rng.integers(lo, mid, n // 2, dtype=dt)
    b = rng.integers(mid, hi, n - n // 2, dtype=dt)
    return np.concatenate([a, b])


def make_ops(rng, scenario, np_variant, B, n):
    """Operation list: a positive entry inserts that many keys, 0 deletes."""
    ops = []
    if scenario == "sort":
        step = B if np_variant else B // 3
        pos = 0
        while pos < n:
            s = min(step, n - pos)
            ops.append(s)
            pos += s
        ops.append(-1)  # marks the end of the insert phase (snapshot)
        ops += [0] * ((n + B - 1) // B + 1)
    elif scenario == "concurrent":
        half = n // 2
        step = B if np_variant else B // 3
        pos = 0
        while pos < half:
            s = min(step, half - pos)
            ops.append(s)
            pos += s
        ops.append(-1)
        step2 = B if np_variant else (2 * B) // 3
        while pos < n:
            s = min(step2, n - pos)
            ops.append(s)
            pos += s
            ops.append(0)
        ops += [0] * ((n + B - 1) // B + 2)
    else:  # mixed (and ties: the same operation mix)
        pos = 0
        while pos < n:
            if rng.random() < 0.65:
                s = B if np_variant else int(rng.integers(1, B + 1))
                s = min(s, n - pos)
                ops.append(s)
                pos += s
            else:
                ops.append(0)
        ops.append(-1)
        ops += [0] * ((n + B - 1) // B + 1)
    return ops


def run_case(ref, variant, kind, scenario, B, seed, rng, nb):
    """Runs one seeded operation sequence through the reference's heap and
    returns (arrays without the case prefix, meta)."""
    np_variant = variant.endswith("_np")
    n = nb * B
    bn = 1
    while bn * B < 2 * n:
        bn <<= 1
    dt, ct, lim = TYPES[kind]
    keys = keys_for(rng, kind, n, scenario == "concurrent", ties=scenario == "ties")
    ops = make_ops(rng, scenario, np_variant, B, n)
    f = lambda name, res=ctypes.c_int: _fn(ref, variant, kind, name, res)
    create = f("create", VP)
    create.argtypes = [ctypes.c_int, ctypes.c_int, ct]
    h = create(bn, B, lim)
    out = np.zeros(n + 2 * B, dt)
    dsizes = []
    sz = ctypes.c_int()
    pos = 0
    snap_items = snap_counters = None
    for op in ops:
        if op > 0:
            chunk = np.ascontiguousarray(keys[pos:pos + op])
            pos += op
            assert f("insert")(VP(h), VP(chunk.ctypes.data), op) == 0
        elif op == 0:
            assert f("delete")(VP(h), VP(out.ctypes.data), ctypes.byref(sz)) == 0
            dsizes.append(sz.value)
        else:
            snap_items = np.zeros((bn + 1) * B, dt)
            snap_counters = np.zeros(3, np.int32)
            f("state")(VP(h), VP(snap_items.ctypes.data), None, VP(snap_counters.ctypes.data))
            assert f("check")(VP(h)) == 1
    items = np.zeros((bn + 1) * B, dt)
    counters = np.zeros(3, np.int32)
    f("state")(VP(h), VP(items.ctypes.data), None, VP(counters.ctypes.data))
    f("destroy", None)(VP(h))
    arrays = dict(keys=keys, ops=np.asarray(ops, np.int32), dsizes=np.asarray(dsizes, np.int32), out=out,
                  snap_items=snap_items, snap_counters=snap_counters, items=items, counters=counters)
    meta = dict(variant=variant, topdown=variant.startswith("td"), partial_buffer=not np_variant, key=kind,
                batch_size=B, batch_num=bn, n=n, scenario=scenario, seed=seed)
    return arrays, meta


def small_cases():
    """48 cases: 4 variants x {u32, u64, i32} x {sort, concurrent, mixed,
    ties} at batch 16-64, 12-26 batches each."""
    for vi, variant in enumerate(VARIANTS):
        for ki, kind in enumerate(["u32", "u64", "i32"]):
            for si, scenario in enumerate(["sort", "concurrent", "mixed", "ties"]):
                seed = 1000 + 97 * vi + 13 * ki + si
                rng = np.random.default_rng(seed)
                B = [16, 32, 64][(vi + ki + si) % 3]
                # an even batch count keeps every insert of the _np variants
                # full: a short insert there pads with init_limits keys that
                # the bottom-up sift-down then chases past the allocation.
                nb = 2 * int(rng.integers(6, 14))
                yield variant, kind, scenario, B, seed, rng, nb


def large_cases():
    """16 cases at the batch sizes of the heap-sort configurations: per
    variant a u32 sort at 2048, a u32 mixed run at 1024, a u64 two-phase
    run at 256 and an i32 tie-heavy run at 512, 4-6 batches each (4 at
    2048)."""
    plan = [("u32", "sort", 2048), ("u32", "mixed", 1024), ("u64", "concurrent", 256), ("i32", "ties", 512)]
    for vi, variant in enumerate(VARIANTS):
        for pi, (kind, scenario, B) in enumerate(plan):
            seed = 5000 + 97 * vi + 13 * pi
            rng = np.random.default_rng(seed)
            nb = 2 * int(rng.integers(2, 4))
            if B == 2048:
                nb = 4  # a three-level heap; keeps the fixture small
            yield variant, kind, scenario, B, seed, rng, nb


def run_retrieve_case(ref, kind, B, seed, rng, n_ops):
    """One seeded sequence of insert(count) / retrieve(size) calls through
    the reference's retrieving heap (applications/sssp_longfei_new/heap.cuh);
    returns (arrays, meta).  ops: positive = insert that many keys, negative
    = retrieve -op keys; `taken` = each retrieve's count, `runs` = the
    retrieved keys, concatenated."""
    dt, ct, lim = TYPES[kind]
    bn = 512
    f = lambda name, res=ctypes.c_int: _fn_rr(ref, kind, name, res)
    create = f("create", VP)
    create.argtypes = [ctypes.c_int, ctypes.c_int, ct]
    h = create(bn, B, lim)
    ops, keys, taken, runs = [], [], [], []
    held = 0
    ties = seed % 3 == 0
    for _ in range(n_ops):
        if rng.random() < 0.55 and held + B < (bn - 8) * B:
            c = int(rng.integers(1, B + 1))
            ks = keys_for(rng, kind, c, False, ties=ties)
            assert f("insert")(VP(h), VP(np.ascontiguousarray(ks).ctypes.data), c) == 0
            ops.append(c)
            keys.append(ks)
            held += c
        else:
            size = int(rng.integers(1, B + 1)) if rng.random() < 0.8 else B
            out = np.zeros(B, dt)
            sz = ctypes.c_int(size)
            assert f("retrieve")(VP(h), VP(out.ctypes.data), ctypes.byref(sz)) == 0
            ops.append(-size)
            taken.append(sz.value)
            runs.append(out[:sz.value].copy())
            held -= sz.value
    # the heap at the end: its valid nodes, the valid part of its partial
    # buffer and {curr_batch_count, curr_pb_size}
    items = np.zeros(bn * B, dt)
    pb = np.zeros(B, dt)
    counters = np.zeros(2, np.int32)
    f("state")(VP(h), VP(items.ctypes.data), VP(pb.ctypes.data), VP(counters.ctypes.data))
    f("destroy", None)(VP(h))
    arrays = dict(ops=np.asarray(ops, np.int32), keys=np.concatenate(keys) if keys else np.zeros(0, dt),
                  taken=np.asarray(taken, np.int32), runs=np.concatenate(runs) if runs else np.zeros(0, dt),
                  final_nodes=items[:int(counters[0]) * B].copy(), final_pb=pb[:int(counters[1])].copy(),
                  final_counters=counters)
    meta = dict(key=kind, batch_size=B, seed=seed, ties=ties, batch_num=bn)
    return arrays, meta


def retrieve_cases():
    """16 sequences of inserts and retrievals: {u32, u64} x batch {16, 64,
    256} x two seeds (every third seed draws keys from ~40 values), then four
    longer u64 sequences at batch 32 and 128 (a deeper heap, every branch of
    retrieve's refill taken many times)."""
    for kind in ("u32", "u64"):
        for B in (16, 64, 256):
            for k in range(2):
                seed = 9000 + 31 * B + 7 * k + (0 if kind == "u32" else 1)
                yield kind, B, seed, np.random.default_rng(seed), 160
    for B in (32, 128):
        for k in range(2):
            seed = 9500 + 13 * B + k
            yield "u64", B, seed, np.random.default_rng(seed), 300


def _fn_rr(lib, kind, name, res):
    fn = getattr(lib, f"rr_{kind}_{name}")
    fn.restype = res
    return fn


def astar_cases():
    """40 seeded bitmaps for the reference's sequential A*
    (artifacts/astar/seq_astar.hpp): sides 1-200, obstacle shares 0-45 %."""
    for k in range(40):
        seed = 12000 + k
        rng = np.random.default_rng(seed)
        w = int(rng.integers(1, 201)) if k >= 4 else [1, 2, 3, 7][k]
        h = int(rng.integers(1, 201)) if k >= 4 else [1, 5, 2, 9][k]
        share = [0.0, 0.1, 0.25, 0.35, 0.45][k % 5]
        yield w, h, share, seed, rng


def run_astar_case(ref, w, h, share, seed, rng):
    """Bitmap (bit i set = cell i open, the corners open) and the reference's
    SeqAstarSearch result on it."""
    open_ = rng.random(w * h) >= share
    open_[0] = open_[-1] = True
    words = np.zeros((w * h + 31) // 32 + 1, np.uint32)
    for i in np.nonzero(open_)[0]:
        words[i // 32] |= np.uint32(1) << np.uint32(i % 32)
    fn = ref.ra_seq_astar
    fn.restype = ctypes.c_uint32
    fn.argtypes = [VP, ctypes.c_uint32, ctypes.c_uint32]
    result = fn(VP(words.ctypes.data), h, w)
    return dict(words=words, result=np.asarray([result], np.uint32)), dict(width=w, height=h, share=share, seed=seed)


SETS = {"small": (small_cases, "bgpq_ref_cases.npz"), "large": (large_cases, "bgpq_ref_cases_large.npz"),
        "retrieve": (retrieve_cases, "retrieve_ref_cases.npz"), "astar": (astar_cases, "astar_ref_cases.npz")}


def main(argv):
    ref = ctypes.CDLL(LIB)
    for name in (argv or ["small", "large", "retrieve", "astar"]):
        gen, fname = SETS[name]
        arrays, meta = {}, []
        for case, params in enumerate(gen()):
            runner = {"retrieve": run_retrieve_case, "astar": run_astar_case}.get(name, run_case)
            a, m = runner(ref, *params)
            arrays.update({f"c{case}_{k}": v for k, v in a.items()})
            meta.append(dict(case=case, **m))
        arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
        path = os.path.join(HERE, fname)
        np.savez_compressed(path, **arrays)
        print(f"wrote {len(meta)} cases to {path} ({os.path.getsize(path)} bytes)")


def _fn(lib, variant, kind, name, res):
    fn = getattr(lib, f"{variant}_{kind}_{name}")
    fn.restype = res
    return fn


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
