"""The batch entry point that allocates nothing (bi_batch_run_noalloc).

Some callers cannot allocate device memory at the point where they run a
batch -- code under an allocator that forbids cudaMalloc, or a callback that
must not allocate.  bi_batch_run_noalloc runs the same uneven batch as a
plan, but keeps its scratch (descriptor copy, work lists, counters) in a
fixed device array owned by the library.  This file checks it against the
allocating path (bi_plan_create + bi_plan_execute) on the same inputs, bit
for bit, on two calls in a row -- the second call finds the array holding
the first call's contents -- and checks that oversized batches are refused.
It is named to run last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream():
    import torch

    return int(torch.cuda.current_stream().cuda_stream)


def test_noalloc_matches_plan_on_two_calls(bigint):
    import torch

    B = bigint
    L = B.lib()
    d, arena, out_limbs, nflags = B.workloads.uneven_batch(n=3000, seed=91, max_bits=32768)
    assert len(d) <= L.bi_batch_noalloc_max_descs()
    din = B.to_device(arena)
    ref_out = torch.zeros(out_limbs, dtype=torch.int64, device="cuda")
    ref_fl = torch.zeros(nflags, dtype=torch.uint8, device="cuda")
    plan = B.Plan(d)
    plan.execute(din, ref_out, ref_fl)
    torch.cuda.synchronize()
    plan.close()
    dp = d.ctypes.data_as(ctypes.c_void_p)
    for call in range(2):
        out = torch.zeros(out_limbs, dtype=torch.int64, device="cuda")
        fl = torch.zeros(nflags, dtype=torch.uint8, device="cuda")
        st = L.bi_batch_run_noalloc(dp, len(d), din.data_ptr(), out.data_ptr(), fl.data_ptr(), _stream())
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
    st = L.bi_batch_run_noalloc(d.ctypes.data_as(ctypes.c_void_p), n, buf.data_ptr(), buf.data_ptr(), None,
                                _stream())
    assert st == 1
    assert b"at most" in L.bi_last_error()
