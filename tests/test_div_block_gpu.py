"""GPU parity of long division against the oracle across the divisor sizes
where the kernels change: the one-limb-per-step warp and lane-group kernels
up to 1024 64-bit limbs, and above that long division KB quotient limbs at a
time on two or four warps (divblock.cuh) up to 4096-limb divisors and
8192-limb dividends -- ragged u32 sizes, divisors shorter than their rows,
dividends that pad the first quotient block, inputs whose block estimate is
capped at B^KB - 1 or one too large (the add-back), zero divisors and
dividends smaller than the divisor, and the 8192 / 4096-limb division of the
largest full product."""
import random

import numpy as np
import pytest

from bigint_gb300.workloads import uniform_limbs

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def _rows(x_list, m, bits=64):
    mask = (1 << bits) - 1
    return np.array([[(x >> (bits * i)) & mask for i in range(m)] for x in x_list],
                    np.uint64 if bits == 64 else np.uint32)


def _run(B, oracle, u, v, method="long"):
    q, r, st = B.div(B.to_device(u), B.to_device(v), method=method)
    q, r, st = B.to_host(q, u.dtype), B.to_host(r, u.dtype), st.cpu().numpy()
    q_ref, r_ref, st_ref = oracle.div(u, v)
    assert (st == st_ref).all()
    bad = np.nonzero(~((q == q_ref).all(1) & (r == r_ref).all(1)))[0]
    assert bad.size == 0, f"{bad.size} mismatching rows, first {bad[:5]}"


# divisor sizes on both sides of each kernel shape: lane groups and warps up
# to 1024 limbs, then the blocked kernel on two warps up to 2048 and four up to 4096
@pytest.mark.parametrize("mv", [129, 200, 256, 257, 400, 512, 513, 777, 1024, 1025, 1500, 2048, 2049, 4096])
def test_shapes_dividend_twice_divisor(bigint, oracle, mv):
    n = 4 if mv > 1024 else 8
    u = uniform_limbs(5100 + mv, n, 2 * mv)
    v = uniform_limbs(5200 + mv, n, mv)
    v[:, -1] |= 1
    u[0] = M64
    v[0] = M64                                    # all ones
    v[1] = 0
    v[1, -1] = 1                                  # B^(mv-1)
    v[2, : mv // 3] = 0                           # a long run of zero low limbs
    _run(bigint, oracle, u, v)


@pytest.mark.parametrize("mu", [1026, 1027, 1029, 1032, 1033, 1034, 1040, 1100, 2500])
def test_first_block_padding(bigint, oracle, mu):
    """1025-limb divisors with dividends whose quotient length takes every
    residue modulo the 8-limb block, from one quotient limb up; and a
    divisor two limbs shorter than its 1025-limb row."""
    mv = 1025
    n = 4
    u = uniform_limbs(5300 + mu, n, mu)
    v = uniform_limbs(5400 + mu, n, mv)
    v[:, -1] |= 1
    u[1, -1] = 0                                  # the top dividend limb zero
    u[2] = M64
    v[3, -2:] = 0
    v[3, -3] |= 1
    _run(bigint, oracle, u, v)


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("mv", [150, 300, 700, 1100, 2500])
def test_short_divisors_in_wide_rows(bigint, oracle, dtype, mv):
    """Rows of mv limbs whose divisor has fewer significant limbs: the shape
    is chosen by the row width, the window by the divisor's precision --
    down to a single limb and to fewer limbs than a quotient block."""
    w = 2 if dtype == np.uint32 else 1
    wv = w * mv - (1 if w == 2 else 0)            # odd u32 word counts
    wu = 2 * wv + 3
    n = 8
    u = uniform_limbs(5700 + mv, n, wu, dtype)
    v = uniform_limbs(5800 + mv, n, wv, dtype)
    for i, keep in enumerate([1, 2, 5, 9, 10, 17, wv // 2, wv - 1]):
        v[i, keep:] = 0
        v[i, keep - 1] |= 1
    _run(bigint, oracle, u, v)


@pytest.mark.parametrize("mu,mv", [(300, 200), (600, 513), (2000, 1024), (3000, 1025), (4200, 2100), (8192, 4096)])
def test_capped_block_estimates(bigint, oracle, mu, mv):
    """u = v B^(mu - mv) - 1 with v's top limb 2^63 over all-ones limbs: every
    quotient limb is B - 1 and the top limbs of the remainder sit just under
    the divisor's, so each block's estimate from the top 2 KB + 1 limbs
    reaches B^KB and is capped."""
    rng = random.Random(mu + mv)
    U, V = [], []
    for variant in range(4):
        if variant == 0:
            v = (1 << (64 * mv - 1)) | ((1 << (64 * (mv - 1))) - 1)
        elif variant == 1:
            v = (1 << (64 * mv)) - 1
        elif variant == 2:
            v = (1 << (64 * mv - 1)) | rng.getrandbits(64 * (mv - 12)) << (64 * 12) | ((1 << (64 * 12)) - 1)
        else:
            v = (1 << (64 * mv - 1)) | ((1 << (64 * mv - 65)) - 1)
        U.append(v * (1 << (64 * (mu - mv))) - 1)
        V.append(v)
    u, v = _rows(U, mu), _rows(V, mv)
    B = bigint
    q, r, st = B.div(B.to_device(u), B.to_device(v), method="long")
    q, r = B.to_host(q, np.uint64), B.to_host(r, np.uint64)
    for i, (x, y) in enumerate(zip(U, V)):
        assert sum(int(a) << (64 * k) for k, a in enumerate(q[i])) == x // y
        assert sum(int(a) << (64 * k) for k, a in enumerate(r[i])) == x % y
    assert (st.cpu().numpy() == 0).all()


@pytest.mark.parametrize("mu,mv", [(260, 130), (1030, 515), (2049, 1030), (4100, 2050), (8192, 4000)])
def test_block_add_back(bigint, oracle, mu, mv):
    """u = (Q v - 1) B^k + low: the block estimate from the top limbs is one
    more than the block's true quotient, so the add-back runs."""
    rng = random.Random(7 * mu + mv)
    U, V = [], []
    for _ in range(4):
        v = rng.getrandbits(64 * mv) | (1 << (64 * mv - 1))
        Qb = rng.getrandbits(64 * 8) | 1
        k = mu - mv - 8
        U.append(((Qb * v - 1) << (64 * k)) | rng.getrandbits(64 * k))
        V.append(v)
    u, v = _rows(U, mu), _rows(V, mv)
    B = bigint
    q, r, st = B.div(B.to_device(u), B.to_device(v), method="long")
    q, r = B.to_host(q, np.uint64), B.to_host(r, np.uint64)
    for i, (x, y) in enumerate(zip(U, V)):
        assert sum(int(a) << (64 * k) for k, a in enumerate(q[i])) == x // y
        assert sum(int(a) << (64 * k) for k, a in enumerate(r[i])) == x % y


@pytest.mark.parametrize("mv", [300, 1024, 3000])
def test_zero_divisor_and_small_dividend(bigint, oracle, mv):
    mu = mv + 40
    u = uniform_limbs(5900 + mv, 5, mu)
    v = uniform_limbs(6000 + mv, 5, mv)
    v[:, -1] |= 1
    v[1] = 0                                       # zero divisor: status 1, q = r = 0
    u[2, mv - 1:] = 0                              # u < v: q = 0, r = u
    u[3] = 0
    _run(bigint, oracle, u, v)


def test_largest_full_product_divides_back(bigint, oracle):
    """An 8192-limb full product of two 4096-limb operands, divided by one of
    them, gives the other and a zero remainder; a product plus a smaller
    remainder gives that remainder back."""
    B = bigint
    n = 2
    a = uniform_limbs(6100, n, 4096)
    b = uniform_limbs(6200, n, 4096)
    b[:, -1] |= 1
    p = B.to_host(B.mulfull(B.to_device(a), B.to_device(b)), np.uint64)
    q, r, st = B.div(B.to_device(p), B.to_device(b))
    q, r = B.to_host(q, np.uint64), B.to_host(r, np.uint64)
    assert (q[:, :4096] == a).all() and (q[:, 4096:] == 0).all() and (r == 0).all()
    _run(bigint, oracle, p, b)


def _pyint_rows(a):
    return [int.from_bytes(row.tobytes(), "little") for row in a]


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
def test_many_instances(bigint, oracle, dtype):
    """Enough 512/256, 2048/1024 and 3000/1500 divisions to fill every warp
    several times: the first 16 rows against the oracle, every row exactly
    in Python integers (u = q v + r, r < v)."""
    B = bigint
    for mv, n in [(256, 3000), (1024, 1400), (1500, 700)]:
        w = 2 if dtype == np.uint32 else 1
        u = uniform_limbs(6300 + mv, n, 2 * mv * w, dtype)
        v = uniform_limbs(6400 + mv, n, mv * w, dtype)
        v[:, -1] |= dtype(1)
        _run(bigint, oracle, u[:16].copy(), v[:16].copy())
        q, r, st = B.div(B.to_device(u), B.to_device(v))
        q, r = B.to_host(q, dtype), B.to_host(r, dtype)
        assert (st.cpu().numpy() == 0).all()
        for x, y, qq, rr in zip(_pyint_rows(u), _pyint_rows(v), _pyint_rows(q), _pyint_rows(r)):
            assert qq * y + rr == x and rr < y
