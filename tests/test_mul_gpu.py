"""GPU parity of batched multiplication (truncated and full product) against
the oracle, including the golden fixtures, the 2048-bit u32 workload with its
all-ones pairs, ragged sizes, the largest supported size, and the full-size
u64 workloads checked on sampled instances."""
import numpy as np
import pytest

from conftest import limbs
from bigint_gb300.workloads import MUL_U64, mul2048_u32, mul_u64_device, splitmix64, uniform_limbs

pytestmark = pytest.mark.gpu


def _both(B, oracle, a, b):
    dt = a.dtype
    da, db = B.to_device(a), B.to_device(b)
    r = B.to_host(B.mul(da, db), dt)
    f = B.to_host(B.mulfull(da, db), dt)
    assert (r == oracle.mul(a, b)).all()
    assert (f == oracle.mulfull(a, b)).all()


def test_golden_fixtures(bigint, oracle, golden):
    B = bigint
    for c in golden["arith"]:
        a, b = limbs(c["a"], c["bits"]), limbs(c["b"], c["bits"])
        da, db = B.to_device(a), B.to_device(b)
        assert (B.to_host(B.mul(da, db), a.dtype) == limbs(c["mul"], c["bits"])).all(), (c["bits"], c["m"])
        assert (B.to_host(B.mulfull(da, db), a.dtype) == limbs(c["mulfull"], c["bits"])).all(), (c["bits"], c["m"])


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("m", [1, 2, 3, 5, 8, 15, 16, 17, 31, 32, 33, 48, 64, 100, 127, 128, 256, 300, 512])
def test_random_parity(bigint, oracle, dtype, m):
    n = max(2, min(300, 40000 // m))
    a = uniform_limbs(41 + m, n, m, dtype)
    b = uniform_limbs(42 + m, n, m, dtype)
    top = np.iinfo(dtype).max
    a[0] = top
    b[0] = top                         # (B^m - 1)^2: every column saturated
    a[1] = 0
    b[1, 0] = 1
    _both(bigint, oracle, a, b)


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
def test_large_sizes(bigint, oracle, dtype):
    L = bigint.lib()
    mmax = int(L.bi_max_limbs_mul_u64() if dtype == np.uint64 else L.bi_max_limbs_mul_u32())
    for m in (1024, 2048, mmax):
        a = uniform_limbs(51 + m, 3, m, dtype)
        b = uniform_limbs(52 + m, 3, m, dtype)
        a[0] = np.iinfo(dtype).max
        b[0] = np.iinfo(dtype).max
        _both(bigint, oracle, a, b)


def test_unsupported_size_rejected(bigint):
    import torch

    B = bigint
    m = int(B.lib().bi_max_limbs_mul_u64()) + 1
    a = torch.zeros((1, m), dtype=torch.int64, device="cuda")
    with pytest.raises(B.BigIntError) as ei:
        B.mulfull(a, a)
    assert ei.value.status == 6


def test_mul2048_u32_workload(bigint, oracle):
    """4096 pairs of 64-limb u32 integers, 10% all-ones; full 128-limb product."""
    a, b = mul2048_u32()
    _both(bigint, oracle, a, b)


def test_host_entry_points(bigint, oracle):
    B = bigint
    for dtype in (np.uint64, np.uint32):
        a = uniform_limbs(61, 77, 40, dtype)
        b = uniform_limbs(62, 77, 40, dtype)
        assert (B.host_mul(a, b) == oracle.mul(a, b)).all()
        assert (B.host_mulfull(a, b) == oracle.mulfull(a, b)).all()


@pytest.mark.parametrize("m,n", MUL_U64)
def test_full_size_workloads(bigint, oracle, m, n):
    """The u64 multiply workloads at full size: sampled exact parity plus the
    truncated product equal to the low half of the full product everywhere."""
    import torch

    B = bigint
    a, b = mul_u64_device(m, n)
    f = B.mulfull(a, b)
    t = B.mul(a, b)
    assert bool((f[:, :m] == t).all())
    idx = np.unique(np.concatenate([(splitmix64(m, 24) % np.uint64(n)).astype(np.int64),
                                    np.array([0, n - 1])]))
    ai = B.to_host(a[idx].contiguous(), np.uint64)
    bi_ = B.to_host(b[idx].contiguous(), np.uint64)
    assert (B.to_host(f[idx].contiguous(), np.uint64) == oracle.mulfull(ai, bi_)).all()
    del a, b, f, t
    torch.cuda.empty_cache()
