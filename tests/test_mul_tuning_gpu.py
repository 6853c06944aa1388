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
    for m, dt in ((64, np.uint64), (100, np.uint64), (256, np.uint64), (200, np.uint32), (16, np.uint64)):
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


def test_autotune_warp_sizes_have_nothing_to_tile(bigint, oracle):
    B = bigint
    a = uniform_limbs(901, 50, 16)
    b = uniform_limbs(902, 50, 16)
    import torch
    da, db = B.to_device(a), B.to_device(b)
    r = torch.zeros((50, 32), dtype=torch.int64, device="cuda")
    assert B.mul_autotune(da, db, r, full=True, reps=1) == (0, 0)
    assert (B.to_host(r, np.uint64) == oracle.mulfull(a, b)).all()
