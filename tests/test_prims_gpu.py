"""GPU parity of the division prototype's helper primitives as batched ops
(bi_cmp, bi_findk, bi_shift, bi_muld, bi_quod) against the oracle's
restatements of prototypes/div.c, on u64 and u32 limbs, random rows and the
edge rows the helpers branch on (equal rows, zero rows, rows that differ only
in the lowest limb, all-ones digits and divisors, zero divisors), and of the
Futhark-shaped 1-D host entries (bi_test_add/sub/mul/div)."""
import numpy as np
import pytest

from bigint_gb300.workloads import uniform_limbs

pytestmark = pytest.mark.gpu

SIZES = [(np.uint64, 1), (np.uint64, 5), (np.uint64, 32), (np.uint64, 33), (np.uint64, 200),
         (np.uint32, 1), (np.uint32, 7), (np.uint32, 64), (np.uint32, 129)]


def _rows(dtype, m, seed, n=64):
    a = uniform_limbs(seed, n, m, dtype)
    b = a.copy()
    top = np.iinfo(dtype).max
    b[0::4, 0] ^= dtype(1)              # differ only in the lowest limb
    b[1::4, m - 1] ^= dtype(1 << 7)     # differ in the top limb
    a[2] = 0                             # zero row
    b[3] = 0
    a[4] = top                           # all ones
    a[5, m // 2:] = 0                    # top half zero
    return a, b


@pytest.mark.parametrize("dtype,m", SIZES)
def test_cmp_and_findk(bigint, oracle, dtype, m):
    B = bigint
    a, b = _rows(dtype, m, 60 + m)
    da, db = B.to_device(a), B.to_device(b)
    assert (B.cmp(da, db).cpu().numpy() == oracle.cmp_rows(a, b)).all()
    assert (B.cmp(db, da).cpu().numpy() == oracle.cmp_rows(b, a)).all()
    assert (B.cmp(da, da).cpu().numpy() == 0).all()
    k, z = B.findk(da)
    kr, zr = oracle.findk_rows(a)
    assert (k.cpu().numpy() == kr).all() and (z.cpu().numpy() == zr).all()


@pytest.mark.parametrize("dtype,m", SIZES)
def test_shift(bigint, oracle, dtype, m):
    B = bigint
    a, _ = _rows(dtype, m, 61 + m)
    da = B.to_device(a)
    for sh in sorted({0, 1, -1, m // 2, -(m // 2), m - 1, -(m - 1), m, -m, m + 3}):
        assert (B.to_host(B.shift(da, sh), dtype) == oracle.shift_rows(a, sh)).all(), sh


@pytest.mark.parametrize("dtype,m", SIZES)
def test_muld_and_quod(bigint, oracle, dtype, m):
    B = bigint
    a, _ = _rows(dtype, m, 62 + m)
    d = uniform_limbs(63 + m, a.shape[0], 1, dtype)[:, 0].copy()
    top = np.iinfo(dtype).max
    d[0] = 0
    d[1] = 1
    d[2] = top
    d[3] = 1 << (8 * np.dtype(dtype).itemsize - 1)   # a normalised divisor already
    d[4] = 3
    d[6] = top                                       # all-ones row by all-ones digit
    a[6] = top
    da, dd = B.to_device(a), B.to_device(d)
    assert (B.to_host(B.muld(da, dd), dtype) == oracle.muld_rows(a, d)).all()
    q, rem = B.quod(da, dd)
    qr, rr = oracle.quod_rows(a, d)
    assert (B.to_host(q, dtype) == qr).all()
    assert (B.to_host(rem, dtype) == rr).all()


def test_futhark_entries(bigint, oracle):
    """bi_test_* = the Futhark library's test_add/sub/mul/div on one integer."""
    import ctypes

    B = bigint
    L = B.lib()
    for dtype, w in ((np.uint64, "u64"), (np.uint32, "u32")):
        for m in (1, 4, 37, 256):
            u = uniform_limbs(64 + m, 1, m, dtype)
            v = uniform_limbs(65 + m, 1, m, dtype)
            v[0, m // 2:] = 0                        # a shorter divisor (equal sizes, leading zeros)
            v[0, 0] |= dtype(1)
            out = np.zeros((1, m), dtype)
            p = lambda x: x.ctypes.data_as(ctypes.c_void_p)
            assert getattr(L, f"bi_test_add_{w}")(p(u), p(v), p(out), m) == 0
            assert (out == oracle.add(u, v)).all()
            assert getattr(L, f"bi_test_sub_{w}")(p(u), p(v), p(out), m) == 0
            assert (out == oracle.sub(u, v)[0]).all()
            assert getattr(L, f"bi_test_mul_{w}")(p(u), p(v), p(out), m) == 0
            assert (out == oracle.mul(u, v)).all()
            assert getattr(L, f"bi_test_div_{w}")(p(u), p(v), p(out), m) == 0
            assert (out == oracle.div(u, v)[0]).all()
            zero = np.zeros((1, m), dtype)
            assert getattr(L, f"bi_test_div_{w}")(p(u), p(zero), p(out), m) == 2   # BI_EDIV0
