"""GPU parity of batched add and sign-magnitude sub against the oracle.

Small and ragged sizes are compared with the oracle in full; the full-size
add/sub sweep (u64, 2^10..2^18 bits, 2^27 limbs per operand) is checked on a
sample of instances against the oracle plus a size-independent property on
every instance: |(a + b) - b| is a when the sum did not wrap and B^m - a when
it did (sign 1), so add(|s - b|, a) == 0 mod B^m exactly for the wrapped rows.
"""
import numpy as np
import pytest

from conftest import limbs
from bigint_gb300.workloads import ADDSUB_BITS, addsub_u64, addsub_u64_device, splitmix64, uniform_limbs

pytestmark = pytest.mark.gpu


def _dev(B, x):
    return B.to_device(x)


def _host(B, t, dtype):
    return B.to_host(t, dtype)


def _check_pair(B, oracle, a, b):
    import torch

    dt = a.dtype
    ra = _host(B, B.add(_dev(B, a), _dev(B, b)), dt)
    assert (ra == oracle.add(a, b)).all()
    rs, sg = B.sub(_dev(B, a), _dev(B, b))
    rs, sg = _host(B, rs, dt), sg.cpu().numpy()
    r_ref, s_ref = oracle.sub(a, b)
    assert (rs == r_ref).all()
    assert (sg == s_ref).all()
    torch.cuda.synchronize()


def test_golden_fixtures(bigint, oracle, golden):
    B = bigint
    for c in golden["arith"]:
        a, b = limbs(c["a"], c["bits"]), limbs(c["b"], c["bits"])
        ra = B.to_host(B.add(B.to_device(a), B.to_device(b)), a.dtype)
        assert (ra == limbs(c["add"], c["bits"])).all(), (c["bits"], c["m"])
        rs, sg = B.sub(B.to_device(a), B.to_device(b))
        assert (B.to_host(rs, a.dtype) == limbs(c["sub"], c["bits"])).all(), (c["bits"], c["m"])
        assert (sg.cpu().numpy() == np.array(c["sign"], np.uint8)).all()


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("m", [1, 2, 3, 5, 7, 8, 16, 31, 33, 64, 100, 128, 255, 512, 1000, 1024,
                               2048, 2049, 4096])
def test_random_parity(bigint, oracle, dtype, m):
    n = max(3, min(700, 200000 // m))
    a = uniform_limbs(31 + m, n, m, dtype)
    b = uniform_limbs(32 + m, n, m, dtype)
    # carry/borrow stress rows: all-ones + 1, equal operands, zero minus one
    top = np.iinfo(dtype).max
    a[0] = top
    b[0] = 0
    b[0, 0] = 1
    b[1] = a[1]
    a[2] = 0
    b[2] = 0
    b[2, 0] = 1
    _check_pair(bigint, oracle, a, b)


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
def test_max_size(bigint, oracle, dtype):
    m = int(bigint.lib().bi_max_limbs_addsub_u64() if dtype == np.uint64
            else bigint.lib().bi_max_limbs_addsub_u32())
    a = uniform_limbs(77, 3, m, dtype)
    b = uniform_limbs(78, 3, m, dtype)
    a[1] = np.iinfo(dtype).max
    b[1] = 0
    b[1, 0] = 1
    _check_pair(bigint, oracle, a, b)


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("m", [3, 16, 64, 513])
@pytest.mark.parametrize("shift_bytes", [8, 16])
def test_unaligned_buffers(bigint, oracle, dtype, m, shift_bytes):
    """Buffers offset by 8 bytes take the scalar path; by 16 bytes, the
    16-byte path even where m would allow the 64-byte-chunk path."""
    import torch

    B = bigint
    n = 97
    a = uniform_limbs(5, n, m, dtype)
    b = uniform_limbs(6, n, m, dtype)
    wide = {np.uint64: torch.int64, np.uint32: torch.int32}[dtype]
    k = shift_bytes // np.dtype(dtype).itemsize
    da = torch.empty(n * m + k, dtype=wide, device="cuda")
    db = torch.empty(n * m + k, dtype=wide, device="cuda")
    dr = torch.empty(n * m + k, dtype=wide, device="cuda")
    da[k:] = B.to_device(a.reshape(-1))
    db[k:] = B.to_device(b.reshape(-1))
    A, Bt, R = da[k:].view(n, m), db[k:].view(n, m), dr[k:].view(n, m)
    B.add(A, Bt, out=R)
    assert (B.to_host(R.contiguous(), dtype) == oracle.add(a, b)).all()
    rs, sg = B.sub(A, Bt, out=R)
    r_ref, s_ref = oracle.sub(a, b)
    assert (B.to_host(R.contiguous(), dtype) == r_ref).all()
    assert (sg.cpu().numpy() == s_ref).all()


def test_in_place_alias(bigint, oracle):
    B = bigint
    a = uniform_limbs(9, 300, 40)
    b = uniform_limbs(10, 300, 40)
    da, db = B.to_device(a), B.to_device(b)
    B.add(da, db, out=da)
    assert (B.to_host(da, np.uint64) == oracle.add(a, b)).all()


def test_host_entry_points(bigint, oracle):
    B = bigint
    for dtype in (np.uint64, np.uint32):
        a = uniform_limbs(21, 513, 24, dtype)
        b = uniform_limbs(22, 513, 24, dtype)
        assert (B.host_add(a, b) == oracle.add(a, b)).all()
        r, s = B.host_sub(a, b)
        r_ref, s_ref = oracle.sub(a, b)
        assert (r == r_ref).all() and (s == s_ref).all()


def test_device_generator_matches_host(bigint):
    t = bigint.workloads.device_uniform_u64(1234, 33, 17, offset=5)
    assert (bigint.to_host(t, np.uint64) == uniform_limbs(1234, 33, 17, offset=5)).all()
    for op in ("add", "sub"):
        a_d, b_d = addsub_u64_device(1 << 11, total_limbs=1 << 14, op=op)
        a_h, b_h = addsub_u64(1 << 11, total_limbs=1 << 14, op=op)
        assert (bigint.to_host(a_d, np.uint64) == a_h).all()
        assert (bigint.to_host(b_d, np.uint64) == b_h).all()


@pytest.mark.parametrize("bits", ADDSUB_BITS)
def test_full_size_sweep(bigint, oracle, bits):
    """2^27 limbs per operand: sampled oracle parity + the wrap property on every row."""
    import torch

    B = bigint
    m = bits // 64
    for op in ("add", "sub"):
        a, b = addsub_u64_device(bits, op=op)
        n = a.shape[0]
        if op == "add":
            r = B.add(a, b)
            s, sign = B.sub(r, b)                      # |(a+b mod B^m) - b|
            back = B.add(s, a)                         # == 0 on wrapped rows
            wrapped = sign.bool()
            ok_plain = (s[~wrapped] == a[~wrapped]).all()
            ok_wrap = (back[wrapped] == 0).all()
            assert bool(ok_plain) and bool(ok_wrap)
        else:
            r, sign = B.sub(a, b)
        # sampled exact parity (chain rows included)
        idx = np.unique(np.concatenate([
            (splitmix64(bits, 256) % np.uint64(n)).astype(np.int64),
            np.arange(min(n, 64)), np.arange(max(0, n - 64), n)]))
        ai = B.to_host(a[idx].contiguous(), np.uint64)
        bi_ = B.to_host(b[idx].contiguous(), np.uint64)
        if op == "add":
            assert (B.to_host(r[idx].contiguous(), np.uint64) == oracle.add(ai, bi_)).all()
        else:
            r_ref, s_ref = oracle.sub(ai, bi_)
            assert (B.to_host(r[idx].contiguous(), np.uint64) == r_ref).all()
            assert (sign[idx].cpu().numpy() == s_ref).all()
        del a, b, r
        torch.cuda.empty_cache()


def test_host_entry_in_place_on_pinned_buffers(bigint, oracle):
    """Pinned host buffers take the in-place path (kernel reads host memory)."""
    import ctypes

    import torch

    B = bigint
    L = B.lib()
    n, m = 1000, 33
    a = uniform_limbs(71, n, m)
    b = uniform_limbs(72, n, m)
    ha = torch.from_numpy(a.view(np.int64)).pin_memory()
    hb = torch.from_numpy(b.view(np.int64)).pin_memory()
    hr = torch.empty_like(ha).pin_memory()
    hs = torch.empty(n, dtype=torch.uint8).pin_memory()
    assert L.bi_host_add_u64(ha.data_ptr(), hb.data_ptr(), hr.data_ptr(), m, n) == 0
    assert (hr.numpy().view(np.uint64) == oracle.add(a, b)).all()
    assert L.bi_host_sub_u64(ha.data_ptr(), hb.data_ptr(), hr.data_ptr(), hs.data_ptr(), m, n) == 0
    r_ref, s_ref = oracle.sub(a, b)
    assert (hr.numpy().view(np.uint64) == r_ref).all() and (hs.numpy() == s_ref).all()
