"""Products of at most 32 64-bit limbs on the per-instance kernels: the
thread kernel (one thread an instance, 64-bit limbs; the default for full
products up to 24 limbs and truncated ones up to 32) and the warp kernel (32-bit words;
full products only, the default from 25 to 32 limbs), each pinned by hand at
every size it takes, both limb widths, against the oracle: saturated
columns, zeros, single bits, ragged last tiles, and a batch larger than one
wave of the thread kernel's grid (the grid-stride loop)."""
import numpy as np
import pytest

from bigint_gb300.workloads import uniform_limbs

pytestmark = pytest.mark.gpu

THREAD_MAX_L = 24
THREAD_TRUNC_MAX_L = 32
WARP_MAX_L = 32


def _limbs64(m, dtype):
    return m if dtype == np.uint64 else (m + 1) // 2


def _cases(seed, n, m, dtype):
    a = uniform_limbs(seed, n, m, dtype)
    b = uniform_limbs(seed + 1, n, m, dtype)
    top = np.iinfo(dtype).max
    a[0] = top
    b[0] = top                                   # (B^m - 1)^2: every column saturated
    a[1] = 0
    a[2] = 0
    a[2, -1] = 1 << (8 * a.itemsize - 1)         # the top bit alone
    b[2] = top
    a[3] = top
    b[3] = 0
    b[3, 0] = 1                                  # times one
    a[4::7] = top                                # saturated rows spread over the tiles
    return a, b


@pytest.fixture(autouse=True)
def _reset(bigint):
    yield
    for m in range(1, 2 * WARP_MAX_L + 1):
        for dt in (np.uint64, np.uint32):
            if _limbs64(m, dt) <= WARP_MAX_L:
                bigint.mul_set_tuning(m, dt, True, 0)
                bigint.mul_set_tuning(m, dt, False, 0)


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("kernel,full", [("default", True), ("thread", True), ("warp", True),
                                         ("default", False), ("thread", False)])
def test_every_small_size(bigint, oracle, dtype, kernel, full):
    B = bigint
    top_m = (THREAD_MAX_L if kernel == "thread" else WARP_MAX_L) if full else THREAD_TRUNC_MAX_L
    sizes = range(1, (top_m if dtype == np.uint64 else 2 * top_m) + 1)
    for m in sizes:
        if kernel != "default":
            B.mul_set_tuning(m, dtype, full, -1, 1 if kernel == "thread" else 0)
        n = 128 + 3 + m                          # one full tile and a ragged one
        a, b = _cases(3000 + m, n, m, dtype)
        da, db = B.to_device(a), B.to_device(b)
        if full:
            assert (B.to_host(B.mulfull(da, db), dtype) == oracle.mulfull(a, b)).all(), (m, dtype, kernel)
        else:
            assert (B.to_host(B.mul(da, db), dtype) == oracle.mul(a, b)).all(), (m, dtype, kernel)
        if kernel != "default":
            B.mul_set_tuning(m, dtype, full, 0)


@pytest.mark.parametrize("full", [True, False])
@pytest.mark.parametrize("m,dtype", [(1, np.uint64), (3, np.uint32), (16, np.uint64), (31, np.uint32), (24, np.uint64),
                                     (47, np.uint32), (32, np.uint64), (63, np.uint32)])
def test_batch_larger_than_the_grid(bigint, m, dtype, full):
    """More instances than the capped grid holds at once (152 SMs x CTAs an SM
    x 128 or 64 instances): rows in every wave, checked as Python integers."""
    B = bigint
    n = 1_300_000 if m <= 3 else 400_000
    a = uniform_limbs(77 + m, n, m, dtype)
    b = uniform_limbs(78 + m, n, m, dtype)
    a[-1] = np.iinfo(dtype).max
    b[-1] = np.iinfo(dtype).max
    da, db = B.to_device(a), B.to_device(b)
    got = B.to_host(B.mulfull(da, db) if full else B.mul(da, db), dtype)
    w = 8 * a.itemsize
    mod = 1 << (w * (2 * m if full else m))

    def val(row):
        return sum(int(x) << (w * k) for k, x in enumerate(row))

    rows = np.unique(np.concatenate([np.arange(0, n, 9973), [n - 129, n - 128, n - 1], np.arange(127, n, 311_296)]))
    for i in rows:
        assert val(got[i]) == val(a[i]) * val(b[i]) % mod, (m, dtype, int(i))


@pytest.mark.parametrize("m", [2, 8, 31, 32, 47, 48])
def test_u32_buffers_off_an_8_byte_boundary(bigint, oracle, m):
    """u32 operands and products starting 4 bytes past an 8-byte boundary: an
    even word count cannot be read as 64-bit limbs there and takes the word
    path; the product is the same."""
    import torch
    B = bigint
    n = 300
    a, b = _cases(5000 + m, n, m, np.uint32)

    def shifted(x):
        buf = torch.zeros(x.size + 1, dtype=torch.int32, device="cuda")
        t = buf[1:].view(x.shape)
        t.copy_(B.to_device(x))
        return t

    da, db = shifted(a), shifted(b)
    rbuf = torch.zeros(n * 2 * m + 1, dtype=torch.int32, device="cuda")
    r = rbuf[1:].view(n, 2 * m)
    assert da.data_ptr() % 8 == 4 and r.data_ptr() % 8 == 4
    B.mulfull(da, db, out=r)
    assert (B.to_host(r, np.uint32) == oracle.mulfull(a, b)).all()
    assert int(rbuf[0]) == 0                                  # nothing written before the product
    tbuf = torch.zeros(n * m + 1, dtype=torch.int32, device="cuda")
    t = tbuf[1:].view(n, m)
    B.mul(da, db, out=t)
    assert (B.to_host(t, np.uint32) == oracle.mul(a, b)).all()
    assert int(tbuf[0]) == 0


def test_pinning_checked(bigint):
    B = bigint
    with pytest.raises(B.BigIntError) as e:
        B.mul_set_tuning(25, np.uint64, True, -1, 1)        # thread kernel above 24 limbs
    assert e.value.status == 1
    with pytest.raises(B.BigIntError):
        B.mul_set_tuning(49, np.uint32, True, -1, 1)        # 25 64-bit limbs
    with pytest.raises(B.BigIntError):
        B.mul_set_tuning(33, np.uint64, True, -1, 0)        # warp kernel above 32 limbs
    with pytest.raises(B.BigIntError):
        B.mul_set_tuning(8, np.uint64, True, -1, 2)         # no such kernel
    with pytest.raises(B.BigIntError):
        B.mul_set_tuning(8, np.uint64, False, -1, 0)        # truncated products: no warp kernel
    with pytest.raises(B.BigIntError):
        B.mul_set_tuning(33, np.uint64, False, -1, 1)       # truncated: thread kernel above 32 limbs
    B.mul_set_tuning(33, np.uint32, True, -1, 0)            # 17 64-bit limbs on the warp kernel: fine
    B.mul_set_tuning(48, np.uint32, True, -1, 1)            # 24 64-bit limbs on the thread kernel: fine
    B.mul_set_tuning(32, np.uint64, False, -1, 1)           # truncated, on the thread kernel: fine
