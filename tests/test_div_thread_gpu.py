"""Long division of divisors up to 16 limbs on one thread an instance
(div_thread_kernel) against the oracle: every divisor size, dividends from
the divisor's size to a few times it, divisors with zero top limbs (a
shorter precision K moves the window), zero divisors, dividends below the
divisor, add-back rows (u = v B^k - 1), ragged last CTAs, and u32 word
counts even, odd and off an 8-byte boundary."""
import numpy as np
import pytest

from bigint_gb300.workloads import uniform_limbs

pytestmark = pytest.mark.gpu


def _inputs(seed, n, mu, mv, dtype):
    u = uniform_limbs(seed, n, mu, dtype)
    v = uniform_limbs(seed + 1, n, mv, dtype)
    top = np.iinfo(dtype).max
    rng = np.random.default_rng(seed)
    for i in range(0, n, 5):                       # shorter divisors: zero top limbs
        k = int(rng.integers(1, mv + 1))
        v[i, k:] = 0
        v[i, k - 1] |= 1
    v[1::11] = top                                 # all-ones divisors, all-ones dividends
    u[1::11] = top
    v[2::13] = 0                                   # zero divisors
    u[3::17] = 0
    u[3::17, 0] = 7                                # dividends below the divisor
    for i in range(4, n, 19):                      # u = v B^k - 1: every estimate on its edge
        k = mu - mv
        vi = sum(int(x) << (8 * v.itemsize * j) for j, x in enumerate(v[i]))
        if vi == 0:
            continue
        ui = min(vi * (1 << (8 * v.itemsize * k)) - 1, (1 << (8 * u.itemsize * mu)) - 1)
        u[i] = [(ui >> (8 * u.itemsize * j)) & int(top) for j in range(mu)]
    return u, v


def _check(B, oracle, u, v):
    q, r, st = B.div(B.to_device(u), B.to_device(v))
    q, r, st = B.to_host(q, u.dtype), B.to_host(r, u.dtype), st.cpu().numpy()
    q_ref, r_ref, st_ref = oracle.div(u, v)
    assert (st == st_ref).all()
    bad = np.nonzero(~((q == q_ref).all(1) & (r == r_ref).all(1)))[0]
    assert bad.size == 0, f"{bad.size} mismatching rows, first {bad[:5]}"


@pytest.mark.parametrize("mv", list(range(1, 17)))
def test_every_divisor_size_u64(bigint, oracle, mv):
    n = 300 if mv <= 8 else 8000                   # above 8 limbs, few instances run on lane groups
    for mu in sorted({mv, mv + 1, 2 * mv, 3 * mv + 2, 47 - (mv | 1)}):
        if mu < mv:
            continue
        _check(bigint, oracle, *_inputs(100 * mv + mu, n, mu, mv, np.uint64))


@pytest.mark.parametrize("mv", [3, 8, 12, 16])
def test_long_dividends(bigint, oracle, mv):
    """Dividends of 45 to 94 limbs over short divisors: long quotients, the
    window sliding through most of the dividend."""
    for mu in (45, 46, 93, 94):
        _check(bigint, oracle, *_inputs(7000 + mu, 7500, mu, mv, np.uint64))


@pytest.mark.parametrize("mw,vw", [(8, 4), (7, 4), (9, 3), (32, 16), (31, 17), (33, 31)])
def test_u32_word_counts(bigint, oracle, mw, vw):
    """Even and odd word counts (a u32 instance is read as the limbs of its
    zero-extended value)."""
    _check(bigint, oracle, *_inputs(900 + mw + vw, 9000, mw, vw, np.uint32))


@pytest.mark.parametrize("mw,vw", [(8, 4), (32, 16)])
def test_u32_off_an_8_byte_boundary(bigint, oracle, mw, vw):
    """u32 operands and results 4 bytes past an 8-byte boundary: the same
    results, nothing written outside them."""
    import torch

    B = bigint
    n = 9000
    u, v = _inputs(950 + mw, n, mw, vw, np.uint32)

    def shifted(x):
        buf = torch.zeros(x.size + 1, dtype=torch.int32, device="cuda")
        t = buf[1:].view(x.shape)
        t.copy_(B.to_device(x))
        return t

    du, dv = shifted(u), shifted(v)
    qb = torch.zeros(n * mw + 1, dtype=torch.int32, device="cuda")
    rb = torch.zeros(n * vw + 1, dtype=torch.int32, device="cuda")
    q, r = qb[1:].view(n, mw), rb[1:].view(n, vw)
    assert du.data_ptr() % 8 == 4 and q.data_ptr() % 8 == 4
    _, _, st = B.div(du, dv, q=q, r=r)
    q_ref, r_ref, st_ref = oracle.div(u, v)
    assert (st.cpu().numpy() == st_ref).all()
    assert (B.to_host(q, np.uint32) == q_ref).all() and (B.to_host(r, np.uint32) == r_ref).all()
    assert int(qb[0]) == 0 and int(rb[0]) == 0


def test_many_ctas(bigint, oracle):
    """Many CTAs with a ragged last one."""
    _check(bigint, oracle, *_inputs(4242, 128 * 300 + 77, 8, 4, np.uint64))
