"""The batch entry point that allocates nothing (bi_batch_run_noalloc).

Some callers cannot allocate device memory at the point where they run a
batch -- code under an allocator that forbids cudaMalloc, or a callback that
must not allocate.  bi_batch_run_noalloc runs the same uneven batch as a
plan, but keeps its scratch (descriptor copy, work lists, counters) in a
fixed device array owned by the library.  This file checks it against the
allocating path (bi_plan_create + bi_plan_execute) bit for bit on two calls
in a row with different batches -- 3000 mixed operations, then 500
divisions only -- so the second call finds the array holding the first
call's descriptors, lists and counters and must not read any of them; and
checks that oversized batches are refused.  It is named to run last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream():
    import torch

    return int(torch.cuda.current_stream().cuda_stream)


def _divisions_only(B, n, seed):
    """n divisions of dividends of 4..300 limbs by divisors of 1..m limbs."""
    rng = np.random.default_rng(seed)
    d = np.zeros(n, dtype=B.DESC_DTYPE)
    pos = out = 0
    for i in range(n):
        m = int(rng.integers(4, 301))
        mb = int(rng.integers(1, m + 1))
        d[i]["op"], d[i]["m"], d[i]["mb"] = B.OP_DIV, m, mb
        d[i]["a"], d[i]["b"] = pos, pos + m
        pos += m + mb
        d[i]["r"], d[i]["r2"] = out, out + m
        out += m + mb
        d[i]["flag"] = i
    arena = rng.integers(0, 2**64, size=pos, dtype=np.uint64)
    for i in range(n):                                   # nonzero top divisor limbs
        arena[d[i]["b"] + d[i]["mb"] - 1] |= np.uint64(1)
    return d, arena, out, n


def _plan_result(B, d, din, out_limbs, nflags):
    import torch

    out = torch.zeros(out_limbs, dtype=torch.int64, device="cuda")
    fl = torch.zeros(nflags, dtype=torch.uint8, device="cuda")
    plan = B.Plan(d, din.numel(), out_limbs, nflags)
    plan.execute(din, out, fl)
    torch.cuda.synchronize()
    plan.close()
    return out, fl


def test_noalloc_matches_plan_on_two_calls(bigint):
    import torch

    B = bigint
    L = B.lib()
    batches = [B.workloads.uneven_batch(n=3000, seed=91, max_bits=32768), _divisions_only(B, 500, 93)]
    for call, (d, arena, out_limbs, nflags) in enumerate(batches):
        assert len(d) <= L.bi_batch_noalloc_max_descs()
        din = B.to_device(arena)
        ref_out, ref_fl = _plan_result(B, d, din, out_limbs, nflags)
        out = torch.zeros(out_limbs, dtype=torch.int64, device="cuda")
        fl = torch.zeros(nflags, dtype=torch.uint8, device="cuda")
        st = L.bi_batch_run_noalloc(d.ctypes.data_as(ctypes.c_void_p), len(d), din.data_ptr(), din.numel(),
                                    out.data_ptr(), out_limbs, fl.data_ptr(), nflags, _stream())
        assert st == 0, L.bi_last_error()
        torch.cuda.synchronize()
        assert bool((out == ref_out).all()), f"call {call}: results differ from bi_plan_execute"
        assert bool((fl == ref_fl).all()), f"call {call}: flags differ from bi_plan_execute"


def test_noalloc_rejects_more_than_its_limit(bigint):
    import torch

    B = bigint
    L = B.lib()
    n = int(L.bi_batch_noalloc_max_descs()) + 1
    d = np.zeros(n, dtype=B.DESC_DTYPE)
    d["m"] = 1
    d["mb"] = 1
    buf = torch.zeros(16, dtype=torch.int64, device="cuda")
    st = L.bi_batch_run_noalloc(d.ctypes.data_as(ctypes.c_void_p), n, buf.data_ptr(), 16, buf.data_ptr(), 16,
                                None, 0, _stream())
    assert st == 1
    assert b"at most" in L.bi_last_error()
