"""The CTA multiply's tilings (instances per CTA, row slices) give the
oracle's products, whether set by hand or picked by the autotuner; the
autotuner leaves r as a plain call writes it and later calls use its choice."""
import numpy as np
import pytest

from bigint_gb300.workloads import uniform_limbs

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _reset(bigint):
    yield
    for m, dt in ((64, np.uint64), (100, np.uint64), (256, np.uint64), (200, np.uint32), (16, np.uint64),
                  (2, np.uint64), (4, np.uint64), (32, np.uint64), (40, np.uint32), (8, np.uint64),
                  (24, np.uint64), (33, np.uint32)):
        for full in (False, True):
            bigint.mul_set_tuning(m, dt, full, 0)


def _check(B, oracle, a, b):
    da, db = B.to_device(a), B.to_device(b)
    assert (B.to_host(B.mul(da, db), a.dtype) == oracle.mul(a, b)).all()
    assert (B.to_host(B.mulfull(da, db), a.dtype) == oracle.mulfull(a, b)).all()


@pytest.mark.parametrize("m,dtype", [(64, np.uint64), (100, np.uint64), (256, np.uint64), (200, np.uint32)])
@pytest.mark.parametrize("ipc,slices", [(1, 1), (1, 2), (1, 4), (2, 2), (4, 1), (3, 2), (8, 4)])
def test_tilings_by_hand(bigint, oracle, m, dtype, ipc, slices):
    B = bigint
    for full in (False, True):
        try:
            B.mul_set_tuning(m, dtype, full, ipc, slices)
        except B.BigIntError as e:
            assert e.status == 1      # does not fit a CTA: refused, nothing set
    n = 37                            # not a multiple of any ipc above
    a = uniform_limbs(500 + m + ipc, n, m, dtype)
    b = uniform_limbs(600 + m + slices, n, m, dtype)
    top = np.iinfo(dtype).max
    a[0] = top
    b[0] = top
    _check(B, oracle, a, b)


@pytest.mark.parametrize("m,dtype", [(64, np.uint64), (256, np.uint64), (200, np.uint32)])
def test_autotune_result_and_later_calls(bigint, oracle, m, dtype):
    B = bigint
    n = 300
    a = uniform_limbs(700 + m, n, m, dtype)
    b = uniform_limbs(800 + m, n, m, dtype)
    for full in (True, False):
        da, db = B.to_device(a), B.to_device(b)
        ipc, slices = B.mul_autotune(da, db, full=full, reps=2)
        assert ipc >= 1 and slices in (1, 2, 4)
        r = B.mulfull(da, db) if full else B.mul(da, db)
        ref = oracle.mulfull(a, b) if full else oracle.mul(a, b)
        assert (B.to_host(r, dtype) == ref).all()


@pytest.mark.parametrize("m,dtype", [(16, np.uint64), (2, np.uint64), (32, np.uint64), (40, np.uint32)])
def test_autotune_weighs_the_warp_kernel_at_small_sizes(bigint, oracle, m, dtype):
    """Full products of at most 32 64-bit limbs: the autotuner times the warp
    kernel (32-bit words, reported as (0, 0)) and, up to 24 limbs, the thread
    kernel (reported as (0, 1)) beside the CTA tilings (64-bit limbs); r and
    every later call are exact whichever wins."""
    B = bigint
    import torch
    n = 500
    a = uniform_limbs(901 + m, n, m, dtype)
    b = uniform_limbs(902 + m, n, m, dtype)
    a[0] = np.iinfo(dtype).max
    b[0] = np.iinfo(dtype).max
    da, db = B.to_device(a), B.to_device(b)
    r = torch.zeros((n, 2 * m), dtype=torch.int64 if dtype == np.uint64 else torch.int32, device="cuda")
    ipc, slices = B.mul_autotune(da, db, r, full=True, reps=2)
    L64 = m if dtype == np.uint64 else (m + 1) // 2
    assert (ipc, slices) == (0, 0) or (L64 <= 24 and (ipc, slices) == (0, 1)) or (ipc >= 1 and slices in (1, 2, 4))
    assert (B.to_host(r, dtype) == oracle.mulfull(a, b)).all()
    assert (B.to_host(B.mulfull(da, db), dtype) == oracle.mulfull(a, b)).all()
    B.mul_set_tuning(m, dtype, True, 0)


@pytest.mark.parametrize("m,dtype", [(8, np.uint64), (24, np.uint64), (33, np.uint32)])
def test_autotune_truncated_small_sizes(bigint, oracle, m, dtype):
    """Truncated products of at most 24 64-bit limbs: the autotuner times the
    thread kernel (reported as (0, 1)) beside the CTA tilings; r and later
    calls are exact whichever wins."""
    import torch

    B = bigint
    n = 700
    a = uniform_limbs(921 + m, n, m, dtype)
    b = uniform_limbs(922 + m, n, m, dtype)
    a[0] = np.iinfo(dtype).max
    b[0] = np.iinfo(dtype).max
    da, db = B.to_device(a), B.to_device(b)
    r = torch.zeros((n, m), dtype=torch.int64 if dtype == np.uint64 else torch.int32, device="cuda")
    ipc, slices = B.mul_autotune(da, db, r, full=False, reps=2)
    assert (ipc, slices) == (0, 1) or (ipc >= 1 and slices in (1, 2, 4))
    assert (B.to_host(r, dtype) == oracle.mul(a, b)).all()
    assert (B.to_host(B.mul(da, db), dtype) == oracle.mul(a, b)).all()


@pytest.mark.parametrize("m", [4, 16, 32])
def test_cta_tiling_by_hand_at_warp_sizes(bigint, oracle, m):
    """A tiling set by hand for a small full product moves it from the thread
    or warp kernel to the CTA kernel; clearing it moves it back; both exact."""
    B = bigint
    n = 77
    a = uniform_limbs(911 + m, n, m)
    b = uniform_limbs(912 + m, n, m)
    da, db = B.to_device(a), B.to_device(b)
    ref = oracle.mulfull(a, b)
    B.mul_set_tuning(m, np.uint64, True, 2, 1)
    assert (B.to_host(B.mulfull(da, db), np.uint64) == ref).all()
    B.mul_set_tuning(m, np.uint64, True, 0)
    assert (B.to_host(B.mulfull(da, db), np.uint64) == ref).all()
