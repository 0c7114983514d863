"""CPU checks of the C ABI library: it loads, exports every entry point that
include/*.h declares, and its pure host calls answer without a GPU."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_entry_points():
    names = set()
    for fn in os.listdir(os.path.join(REPO, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(REPO, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(gh_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_entry_points()
    assert "gh_heap_create" in names and "gh_heap_sort" in names and len(names) >= 20


@pytest.mark.parametrize("name", declared_entry_points())
def test_library_exports(ghlib, name):
    assert hasattr(ghlib, name), f"{name} declared in include/ but not exported"


def test_python_binding_covers_header(ghlib):
    import gpuheap_gb300 as gh
    missing = set(declared_entry_points()) - set(gh._SIGS)
    assert not missing, f"no ctypes signature for {sorted(missing)}"


def test_host_only_calls(ghlib):
    import gpuheap_gb300 as gh
    assert ghlib.gh_status_string(gh.GH_ERR_TIMEOUT) == b"device wait timed out"
    assert ghlib.gh_heap_view_bytes() == 64
    # 4 node buffers of B keys + 128 bytes of control + 16 of alignment slack
    assert ghlib.gh_heap_smem_bytes(0, 1024) == 4 * 1024 * 4 + 144
    assert ghlib.gh_heap_smem_bytes(2, 1024) == 4 * 1024 * 8 + 144


def test_rejects_bad_arguments_before_touching_a_device(ghlib):
    h = ctypes.c_void_p()
    assert ghlib.gh_heap_create(ctypes.byref(h), 0, 0, 1, 16, 100, None) == 1   # batch size not a power of 2
    assert ghlib.gh_heap_create(ctypes.byref(h), 9, 0, 1, 16, 128, None) == 1   # key kind
    assert ghlib.gh_heap_create(ctypes.byref(h), 0, 5, 1, 16, 128, None) == 1   # variant
    assert ghlib.gh_heap_create(None, 0, 0, 1, 16, 128, None) == 1
    assert ghlib.gh_heap_insert(None, None, 0, 0, None) == 1
    assert ghlib.gh_heap_concurrent(None, None, 0, 0, None, 0, None, None) == 1
    assert ghlib.gh_batch_create(None, 256, 1, 0) == 1
    assert ghlib.gh_batch_destroy(None) == 1
    assert ghlib.gh_batch_build(None, None) == 1
    assert ghlib.gh_batch_run(None, 0, None) == 1
    assert ghlib.gh_batch_add_astar(None, 4, 4, None, None) == 1
    assert ghlib.gh_gen_grid(0, 4, 1, 200, None, 1) == 1
    assert ghlib.gh_serve_create(None, 0, 4, 256, 1, 8) == 1
    assert ghlib.gh_serve_destroy(None) == 1
    assert ghlib.gh_serve_step(None, None, None, None, None) == 1
    assert ghlib.gh_serve_submit(None, 2, 0, 0, 0, None) == 1
    assert ghlib.gh_heap_sort_host(None, None, 0, None, None) == 1
    assert ghlib.gh_rheap_create(None, 2, 64, 64, None) == 1
    assert ghlib.gh_rheap_destroy(None) == 1
    assert ghlib.gh_rheap_insert(None, None, 1, None) == 1
    assert ghlib.gh_rheap_retrieve(None, None, None, None) == 1
    assert ghlib.gh_rheap_state(None, None, None, None) == 1
    assert ghlib.gh_sssp_retrieve(0, None, None, None, 0, None, 64, 8, 1, 0, None, None) == 1
    assert ghlib.gh_serve_start(None, 100) == 1
    assert ghlib.gh_serve_poll(None, None, None, None) == 1
    assert ghlib.gh_serve_stop(None) == 1


def test_newer_entry_points_reject_bad_arguments(ghlib):
    """Delete below a threshold, GC, retrieval, single-block operations,
    launch-shape setters and the knapsack order refuse a missing handle or
    threshold with GH_ERR_INVALID, before any device work."""
    t = ctypes.c_uint32(5)
    n = ctypes.c_longlong()
    sz = ctypes.c_int()
    assert ghlib.gh_heap_delete_below(None, None, 0, ctypes.byref(t), ctypes.byref(n), None) == 1
    assert ghlib.gh_heap_delete_below(None, None, 0, None, ctypes.byref(n), None) == 1      # no threshold
    assert ghlib.gh_heap_gc(None, ctypes.byref(t), ctypes.byref(n), None) == 1
    assert ghlib.gh_heap_retrieve(None, None, 0, ctypes.byref(sz), None) == 1
    assert ghlib.gh_heap_insert_batch(None, None, 1, None) == 1
    assert ghlib.gh_heap_delete_batch(None, None, ctypes.byref(sz), None) == 1
    assert ghlib.gh_heap_set_timeout(None, 1.0) == 1
    assert ghlib.gh_heap_set_block_threads(None, 0) == 1
    assert ghlib.gh_heap_set_grid(None, 0) == 1
    assert ghlib.gh_heap_inject_lock(None, 0, 1) == 1
    assert ghlib.gh_batch_set_knapsack_order(None, 0, 20) == 1
    assert ghlib.gh_batch_knapsack_switches(None, None, None) == 1
    assert ghlib.gh_batch_set_astar_blocks(None, 1 << 18, 8) == 1
    assert ghlib.gh_batch_set_timeout(None, 1.0) == 1
    assert ghlib.gh_serve_set_blocks(None, 1 << 15, 24, 1 << 18, 8) == 1
    cnt = (ctypes.c_int * 3)(0, 0, 0)
    assert ghlib.gh_heap_restore(None, ctypes.byref(t), cnt) == 1


def test_primitive_and_owner_entry_points_reject_bad_arguments(ghlib):
    """The block-primitive entry points, the owner-mode depth setter and the
    owner counters refuse bad shapes or a missing handle with GH_ERR_INVALID
    before any device work."""
    p = ctypes.c_void_p(16)  # never dereferenced: the checks come first
    assert ghlib.gh_merge_batches(0, 0, p, p, 100, p, p, 128, None) == 1      # n not a power of two
    assert ghlib.gh_merge_batches(0, 0, p, p, 2048, p, p, 32, None) == 1      # 128 keys per thread
    assert ghlib.gh_merge_batches(0, 1, p, p, 256, p, p, 256, None) == 1      # below one 1024-key window
    assert ghlib.gh_merge_batches(0, 2, p, p, 256, p, p, 256, None) == 1      # no such method
    assert ghlib.gh_merge_batches(3, 0, p, p, 256, p, p, 256, None) == 1      # no such key kind
    assert ghlib.gh_merge_batches(0, 0, None, p, 256, p, p, 256, None) == 1
    assert ghlib.gh_sort_batch(0, p, 100, p, 128, None) == 1
    assert ghlib.gh_sort_batch(0, p, 256, p, 48, None) == 1
    assert ghlib.gh_heap_set_owner_depth(None, 2) == 1
    out = (ctypes.c_ulonglong * 4)()
    assert ghlib.gh_heap_owner_stats(None, out, 4) == 1
