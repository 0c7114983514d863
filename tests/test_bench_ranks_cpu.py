"""The multi-rank path of bench.py on CPU: two gloo ranks agree on the
slowest rank's time (the contract's max over ranks), the whole-job rate
counts every rank's keys, and the reference arm prints from rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, REPO)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        rate = bench.job_rate(1 << 20, world, 3, ms)
        q.put((rank, ms, rate))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [15.0, 15.0]          # both ranks see the slowest
    want = (1 << 20) * 2 * 3 / 0.015 / 1e6               # every rank's keys / the max time
    assert all(abs(g[2] - want) < 1e-9 * want for g in got)


def test_single_rank_helpers():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert abs(bench.job_rate(1000, 1, 2, 4.0) - 0.5) < 1e-12


def test_reference_arm_prints_from_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_line_on_one_rank():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-sample-log2", "18"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_roofline_traffic_is_the_capture_for_the_exact_workload():
    """roofline.traffic is the ncu DRAM read+write of one launch of the
    bench's own workload (profiles/traffic.json) and null for any other
    size, layout or launch shape -- it is never scaled from another size."""
    sys.path.insert(0, REPO)
    import bench
    sys_argv, sys.argv = sys.argv, ["bench.py"]
    try:
        a = bench.parse()
    finally:
        sys.argv = sys_argv
    with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
        d = json.load(f)
    e = d["k_delete_owner/bottomup/pb/B2048/u32/uniform/2^28"]
    assert bench.ncu_traffic("k_delete_owner", a, True) == e["read"] + e["write"]
    assert bench.ncu_traffic("k_insert_reserved", a, True) > 0
    assert bench.ncu_traffic("k_delete_owner", a, False) is None
    a.log2n = 25
    assert bench.ncu_traffic("k_delete_owner", a, True) is None
    a.log2n, a.grid = 28, 76
    assert bench.ncu_traffic("k_delete_owner", a, True) is None
