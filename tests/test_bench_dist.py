"""The bench's multi-rank path on CPU with the gloo backend (world size 2):
every rank runs the full workload, the timed region is the maximum over
ranks, and the whole-job rate counts every rank's bytes; the reference arm
prints from rank 0 only."""
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
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # rank r measured 10 + r ms for a step of 1 GB, 2 steps
        q.put((rank, bench.whole_job(10.0 + rank, 10**9, 2, world)))
    finally:
        dist.destroy_process_group()


def test_whole_job_rate_is_max_over_ranks_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        ms, gbs = got[r]
        assert ms == 11.0                                   # the slower rank's time, on both ranks
        assert abs(gbs - 2 * 10**9 * 2 / 0.011 / 1e9) < 1e-6   # both ranks' bytes in that time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench

    ms, gbs = bench.whole_job(4.0, 3 * 10**9, 5, 1)
    assert ms == 4.0 and abs(gbs - 3 * 5 / 0.004) < 1e-6


def test_reference_arm_prints_from_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_gu32ops_follows_the_reference_formula():
    # cuda/main.cu:393-400: num_instances * 300 * M * log2(M) u32 ops over the elapsed microseconds * 1000
    sys.path.insert(0, REPO)
    import bench

    n, words, ms = 4096, 128, 0.5
    assert abs(bench.gu32ops(n, words, ms) - n * 300 * words * 7 / (ms * 1000 * 1000)) < 1e-9
    assert bench.gu32ops(1, 2, 1e-6) == 300 * 2 * 1   # log2(2) = 1


def test_bench_division_method_follows_the_library_rule():
    """bench.div_method (which method's limb products a division rate is
    counted in) restates div_small_on_groups / div_use_long of divsmall.cuh;
    the thresholds are read from that header so that the two cannot drift."""
    import re

    sys.path.insert(0, REPO)
    import bench

    src = open(os.path.join(REPO, "big-int_gb300", "csrc", "divsmall.cuh")).read()
    group_per_sm = int(re.search(r"DIV_SMALL_GROUP_PER_SM\s*=\s*(\d+)", src).group(1))
    thread_max = int(re.search(r"DIV_THREAD_MAX_MV\s*=\s*(\d+)", src).group(1))
    long_all = int(re.search(r"if \(MV <= (\d+)\) return true;", src).group(1))
    m = re.search(r"per_sm = MV <= 128 \? (\d+) : MV <= 256 \? (\d+) : MV <= 512 \? (\d+) : (\d+);", src)
    per_sm = [int(x) for x in m.groups()]

    def rule(mv, n, sms):
        if mv <= thread_max:
            return "long_group" if mv > 8 and n <= group_per_sm * sms else "long_thread"
        if mv <= long_all:
            return "long_group"
        if mv <= 1024:
            k = per_sm[0] if mv <= 128 else per_sm[1] if mv <= 256 else per_sm[2] if mv <= 512 else per_sm[3]
            if n > k * sms:
                return "long_group"
        return "shinv"

    for sms in (152, 148):
        for mv in (1, 4, 8, 9, 16, 17, 32, 64, 65, 128, 129, 256, 257, 512, 513, 1024, 1025):
            for n in (1, 100, 300, 456, 457, 608, 609, 760, 761, 912, 913, 1520, 7296, 7297, 20000):
                assert bench.div_method(mv, n, sms) == rule(mv, n, sms), (mv, n, sms)
