"""GPU parity of batched division (quotient and remainder) against the
oracle: the golden fixtures and the reference's known-answer vectors, the
divisor-precision sweep of prototypes/div.c:509-523, special divisors
(B^k, B^k - 1, B^k + 1, single limb), shorter divisors, zero divisors, and
the dividend-2m / divisor-m shape of the uneven-batch workload."""
import numpy as np
import pytest

from conftest import limbs
from bigint_gb300.workloads import splitmix64, uniform_limbs

pytestmark = pytest.mark.gpu


def _run(B, oracle, u, v):
    q, r, st = B.div(B.to_device(u), B.to_device(v))
    q, r, st = B.to_host(q, u.dtype), B.to_host(r, u.dtype), st.cpu().numpy()
    q_ref, r_ref, st_ref = oracle.div(u, v)
    assert (st == st_ref).all()
    bad = np.nonzero(~((q == q_ref).all(1) & (r == r_ref).all(1)))[0]
    assert bad.size == 0, f"{bad.size} mismatching rows, first {bad[:5]}"


def test_golden_fixtures(bigint, golden):
    B = bigint
    for c in golden["div"]:
        u, v = limbs(c["u"], c["bits"]), limbs(c["v"], c["bits"])
        q, r, st = B.div(B.to_device(u), B.to_device(v))
        assert (B.to_host(q, u.dtype) == limbs(c["q"], c["bits"])).all(), (c["bits"], c["mu"], c["mv"])
        assert (B.to_host(r, u.dtype) == limbs(c["r"], c["bits"])).all(), (c["bits"], c["mu"], c["mv"])
        assert (st.cpu().numpy() == 0).all()


def test_reference_kats(bigint, golden):
    B = bigint
    for k in golden["kat"]:
        u, v = limbs([k["u"]], 32), limbs([k["v"]], 32)
        q, r, _ = B.div(B.to_device(u), B.to_device(v))
        assert [int(x) for x in B.to_host(q, np.uint32)[0]] == k["q"], k["source"]
        assert [int(x) for x in B.to_host(r, np.uint32)[0]] == k["r"], k["source"]


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 8, 13, 16, 31, 32, 33, 64, 100])
def test_divisor_precision_sweep(bigint, oracle, dtype, m):
    """Equal sizes, divisor precision 1..m as in prototypes/div.c:509-523."""
    n = 3 * m
    u = uniform_limbs(101 + m, n, m, dtype)
    v = uniform_limbs(102 + m, n, m, dtype)
    for i in range(n):
        v[i, 1 + i % m:] = 0
        if v[i, 0] == 0:
            v[i, 0] = 1
    _run(bigint, oracle, u, v)


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("mv", [1, 2, 7, 16, 50, 128, 512])
def test_dividend_twice_divisor(bigint, oracle, dtype, mv):
    """The uneven-batch division shape: dividend 2m limbs, divisor m limbs with a nonzero top limb."""
    n = max(4, min(64, 4000 // mv))
    u = uniform_limbs(201 + mv, n, 2 * mv, dtype)
    v = uniform_limbs(202 + mv, n, mv, dtype)
    v[:, -1] |= 1
    top = np.iinfo(dtype).max
    u[0] = top
    v[0] = top
    u[1] = top
    v[1] = 0
    v[1, -1] = 1                       # v = B^(m-1)
    v[2] = 0
    v[2, 0] = 1
    v[2, -1] = 1                       # v = B^(m-1) + 1
    _run(bigint, oracle, u, v)


def test_special_values(bigint, oracle):
    m = 6
    rows_u, rows_v = [], []
    B64 = 1 << 64
    vals = [(0, 5), (7, 7), (6, 7), (B64**6 - 1, 1), (B64**6 - 1, B64 - 1), (B64**6 - 1, B64**3),
            (B64**6 - 1, B64**3 - 1), (B64**6 - 1, B64**3 + 1), (B64**5, B64**5 - 1), (B64**6 - 1, B64**6 - 1),
            (B64**6 - 2, B64**6 - 1), (3 * B64**4 + 11, 2 * B64 + 1), (B64**6 - 1, 1 << 63), (12345, 1 << 200)]
    for x, y in vals:
        rows_u.append([(x >> (64 * i)) & (B64 - 1) for i in range(m)])
        rows_v.append([(y >> (64 * i)) & (B64 - 1) for i in range(m)])
    _run(bigint, oracle, np.array(rows_u, np.uint64), np.array(rows_v, np.uint64))


def test_zero_divisor_flagged(bigint, oracle):
    B = bigint
    u = uniform_limbs(7, 5, 4)
    v = uniform_limbs(8, 5, 4)
    v[2] = 0
    q, r, st = B.div(B.to_device(u), B.to_device(v))
    st = st.cpu().numpy()
    assert list(st) == [0, 0, 1, 0, 0]
    assert (B.to_host(q, np.uint64)[2] == 0).all() and (B.to_host(r, np.uint64)[2] == 0).all()
    with pytest.raises(B.BigIntError) as ei:
        B.host_div(u, v)
    assert ei.value.status == 2


@pytest.mark.parametrize("mv", [256, 1024])
def test_large_divisions(bigint, oracle, mv):
    n = 3
    u = uniform_limbs(301 + mv, n, 2 * mv)
    v = uniform_limbs(302 + mv, n, mv)
    v[:, -1] |= 1
    _run(bigint, oracle, u, v)


def test_host_entry(bigint, oracle):
    B = bigint
    for dtype in (np.uint64, np.uint32):
        u = uniform_limbs(401, 33, 12, dtype)
        v = uniform_limbs(402, 33, 5, dtype)
        v[:, -1] |= 1
        q, r, st = B.host_div(u, v)
        q_ref, r_ref, _ = oracle.div(u, v)
        assert (q == q_ref).all() and (r == r_ref).all() and (st == 0).all()


def test_exact_where_reference_prototype_is_one_short(bigint, oracle):
    """prototypes/div.c returns q one short (r >= v) on this input; the GPU
    division returns the exact quotient and remainder."""
    U, V = 0xdc4461359674c9cfd718dc1b567834b5, 0xdd2982a538271953
    u = np.array([[(U >> (32 * i)) & 0xFFFFFFFF for i in range(4)]], np.uint32)
    v = np.array([[(V >> (32 * i)) & 0xFFFFFFFF for i in range(2)]], np.uint32)
    q, r, st = bigint.div(bigint.to_device(u), bigint.to_device(v))
    qv = bigint.to_host(q, np.uint32)[0]
    rv = bigint.to_host(r, np.uint32)[0]
    assert sum(int(x) << (32 * i) for i, x in enumerate(qv)) == U // V
    assert sum(int(x) << (32 * i) for i, x in enumerate(rv)) == U % V
    qf, _, _ = oracle.div_ref(u, np.array([[*v[0], 0, 0]], np.uint32))
    assert sum(int(x) << (32 * i) for i, x in enumerate(qf[0])) == U // V - 1
