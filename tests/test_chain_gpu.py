"""GPU parity of the fused chains (bi_add_chain_*, bi_mul_chain_*), the
reference's second benchmark type: p chained additions r1 = a + b, then
r = r1 + r (baddKer1Bench, the thesis's 10(u+v)), and p chained truncated
multiplications
r1 = a b, then r = r1 r (convMul5Bench), each against the oracle's single
operations applied p times.  Sizes that take the fused kernels and sizes
that fall back to separate launches; u64 and u32; odd u32 sizes (the
truncation to m words between steps)."""
import numpy as np
import pytest

from bigint_gb300.workloads import uniform_limbs

pytestmark = pytest.mark.gpu


def _add_chain_ref(oracle, a, b, p):
    r1 = oracle.add(a, b)
    r = r1
    for _ in range(p - 1):
        r = oracle.add(r1, r)
    return r


def _mul_chain_ref(oracle, a, b, p):
    r1 = oracle.mul(a, b)
    r = r1
    for _ in range(p - 1):
        r = oracle.mul(r1, r)
    return r


@pytest.mark.parametrize("dtype,m", [(np.uint64, 8), (np.uint64, 16), (np.uint64, 64), (np.uint64, 100),
                                     (np.uint64, 2048), (np.uint64, 4096), (np.uint64, 8192),
                                     (np.uint32, 16), (np.uint32, 37), (np.uint32, 512)])
@pytest.mark.parametrize("p", [1, 2, 10])
def test_add_chain(bigint, oracle, dtype, m, p):
    B = bigint
    n = max(3, min(400, 100000 // m))
    a = uniform_limbs(40 + m, n, m, dtype)
    b = uniform_limbs(41 + m, n, m, dtype)
    top = np.iinfo(dtype).max
    a[0] = top                  # carry through every limb
    b[0] = 0
    b[0, 0] = 1
    a[1] = top >> 1             # a + b doubles into the top bit
    b[1] = 0
    r = B.to_host(B.add_chain(B.to_device(a), B.to_device(b), p), dtype)
    assert (r == _add_chain_ref(oracle, a, b, p)).all()


@pytest.mark.parametrize("dtype,m", [(np.uint64, 1), (np.uint64, 3), (np.uint64, 16), (np.uint64, 64),
                                     (np.uint64, 100), (np.uint64, 256), (np.uint32, 1), (np.uint32, 7),
                                     (np.uint32, 64), (np.uint32, 129)])
@pytest.mark.parametrize("p", [1, 2, 6])
def test_mul_chain(bigint, oracle, dtype, m, p):
    B = bigint
    n = max(3, min(300, 20000 // m))
    a = uniform_limbs(50 + m, n, m, dtype)
    b = uniform_limbs(51 + m, n, m, dtype)
    a[0] = np.iinfo(dtype).max
    b[0] = np.iinfo(dtype).max
    r = B.to_host(B.mul_chain(B.to_device(a), B.to_device(b), p), dtype)
    assert (r == _mul_chain_ref(oracle, a, b, p)).all()


def test_chain_rejects_zero_steps(bigint):
    import ctypes

    import torch

    B = bigint
    a = torch.zeros((4, 8), dtype=torch.int64, device="cuda")
    with pytest.raises(B.BigIntError):
        B.add_chain(a, a, 0)
    with pytest.raises(B.BigIntError):
        B.mul_chain(a, a, 0)
    assert B.lib().bi_add_chain_u64(ctypes.c_void_p(0x1000), ctypes.c_void_p(0x1000), None, 8, 4, 1, None) == 1
