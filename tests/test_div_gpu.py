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


def _run(B, oracle, u, v, method="auto"):
    q, r, st = B.div(B.to_device(u), B.to_device(v), method=method)
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


@pytest.mark.parametrize("method", ["auto", "shinv", "long"])
@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("m", [1, 2, 3, 4, 5, 8, 13, 16, 17, 31, 32, 33, 64, 100])
def test_divisor_precision_sweep(bigint, oracle, dtype, m, method):
    """Equal sizes, divisor precision 1..m as in prototypes/div.c:509-523."""
    n = 3 * m
    u = uniform_limbs(101 + m, n, m, dtype)
    v = uniform_limbs(102 + m, n, m, dtype)
    for i in range(n):
        v[i, 1 + i % m:] = 0
        if v[i, 0] == 0:
            v[i, 0] = 1
    _run(bigint, oracle, u, v, method)


@pytest.mark.parametrize("method", ["auto", "shinv", "long"])
@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("mv", [1, 2, 7, 16, 50, 128, 512])
def test_dividend_twice_divisor(bigint, oracle, dtype, mv, method):
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
    _run(bigint, oracle, u, v, method)


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


@pytest.mark.parametrize("method", ["auto", "shinv", "long"])
@pytest.mark.parametrize("mv", [256, 1024])
def test_large_divisions(bigint, oracle, mv, method):
    n = 3
    u = uniform_limbs(301 + mv, n, 2 * mv)
    v = uniform_limbs(302 + mv, n, mv)
    v[:, -1] |= 1
    _run(bigint, oracle, u, v, method)


@pytest.mark.parametrize("mu,mv", [(16, 16), (17, 17), (40, 32), (40, 33), (2048, 1024), (2048, 1025), (2048, 2048)])
def test_method_boundaries(bigint, oracle, mu, mv):
    """Divisor sizes on either side of the method limits (16 and 128 64-bit
    limbs for the thread and warp long divisions) and the shifted inverse's
    largest dividend, by every method."""
    n = 3
    u = uniform_limbs(311 + mv, n, mu)
    v = uniform_limbs(312 + mv, n, mv)
    v[:, -1] |= 1
    v[1, mv // 2:] = 0                 # shorter divisor in a wider row
    v[1, mv // 2 - 1] |= 1
    for method in ("auto", "shinv", "long"):
        _run(bigint, oracle, u, v, method)


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("method,n", [("long", 37), ("auto", 1000)])
def test_lane_width_boundaries(bigint, dtype, method, n):
    """Divisors on either side of each lane width of long division -- 16-lane
    groups of 24 and 32 limbs (up to 384 and 512 limbs), warps of 20, 24, 28
    and 32 limbs a lane (up to 640, 768, 896 and 1024) -- with 2m-limb dividends, shorter
    divisors in a wider row, all-ones operands and dividends below the
    divisor; checked as Python integers (u = q v + r, r < v)."""
    B = bigint
    w = 2 if dtype == np.uint32 else 1
    bits = 8 * np.dtype(dtype).itemsize
    for mv in (256, 257, 320, 321, 384, 385, 448, 449, 512, 513, 640, 641, 768, 769, 896, 897, 1024):
        u = uniform_limbs(700 + mv, n, 2 * mv * w, dtype)
        v = uniform_limbs(701 + mv, n, mv * w, dtype)
        v[:, -1] |= 1
        v[1, (mv * w) // 2:] = 0
        v[1, (mv * w) // 2 - 1] |= 1
        u[2] = np.iinfo(dtype).max
        v[2] = np.iinfo(dtype).max
        u[3, mv * w:] = 0                          # u < v
        q, r, st = B.div(B.to_device(u), B.to_device(v), method=method)
        q, r = B.to_host(q, dtype), B.to_host(r, dtype)
        assert (st.cpu().numpy() == 0).all()
        for i in range(n):
            U = int.from_bytes(u[i].tobytes(), "little")
            V = int.from_bytes(v[i].tobytes(), "little")
            Q = int.from_bytes(q[i].tobytes(), "little")
            R = int.from_bytes(r[i].tobytes(), "little")
            assert Q * V + R == U and R < V, (mv, i, bits)


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
def test_small_lane_shape_boundaries(bigint, dtype):
    """Divisors on either side of the lane-group shapes below 256 limbs (8-lane
    groups of 4, 6, 8 limbs up to 32, 48, 64; 16-lane groups of 6 and 8 up to
    96 and 128; warps of 6 and 8 up to 192 and 256), with enough instances
    (2000) that the groups run; checked as Python integers."""
    B = bigint
    w = 2 if dtype == np.uint32 else 1
    n = 2000
    for mv in (17, 24, 25, 32, 33, 48, 49, 64, 65, 96, 97, 128, 129, 192, 193):
        u = uniform_limbs(800 + mv, n, 2 * mv * w, dtype)
        v = uniform_limbs(801 + mv, n, mv * w, dtype)
        v[:, -1] |= 1
        v[1::9, (mv * w) // 2:] = 0
        v[1::9, (mv * w) // 2 - 1] |= 1
        u[2::13] = np.iinfo(dtype).max
        v[2::13] = np.iinfo(dtype).max
        q, r, st = B.div(B.to_device(u), B.to_device(v), method="long")
        q, r = B.to_host(q, dtype), B.to_host(r, dtype)
        assert (st.cpu().numpy() == 0).all()
        for i in range(0, n, 7):
            U = int.from_bytes(u[i].tobytes(), "little")
            V = int.from_bytes(v[i].tobytes(), "little")
            Q = int.from_bytes(q[i].tobytes(), "little")
            R = int.from_bytes(r[i].tobytes(), "little")
            assert Q * V + R == U and R < V, (mv, i)


def test_size_limits_rejected(bigint):
    """Dividends above 8192 64-bit limbs, shifted-inverse dividends above 2048
    and long-division divisors above 4096 are refused before any launch."""
    import torch

    B = bigint
    for mu, mv, method in [(8193, 4, "auto"), (2049, 1000, "shinv"), (8192, 4097, "long")]:
        u = torch.zeros((1, mu), dtype=torch.int64, device="cuda")
        v = torch.ones((1, mv), dtype=torch.int64, device="cuda")
        with pytest.raises(B.BigIntError) as ei:
            B.div(u, v, method=method)
        assert ei.value.status == 6            # BI_EUNSUPPORTED


@pytest.mark.parametrize("method", ["auto", "long", "shinv"])
@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("mu,mv", [(2048, 1), (1000, 3), (700, 16), (700, 17), (1999, 40), (1500, 100), (2048, 513)])
def test_long_dividend_short_divisor(bigint, oracle, dtype, mu, mv, method):
    """Dividends many times longer than the divisor: the long divisions stream
    hundreds of dividend limbs through their window (the warp kernel reloads
    its 32-limb buffer dozens of times), with ragged u32 sizes."""
    if dtype == np.uint32:
        mu, mv = 2 * mu - 1, 2 * mv - 1     # odd word counts: a half-filled top 64-bit limb
    n = 6
    u = uniform_limbs(1300 + mu, n, mu, dtype)
    v = uniform_limbs(1400 + mv, n, mv, dtype)
    v[:, -1] |= 1
    top = np.iinfo(dtype).max
    u[0] = top
    v[0] = top                         # all-ones operands
    u[1, mu // 2:] = 0                 # a dividend half as long
    v[2, :] = 0
    v[2, 0] = 1                        # v = 1: q = u
    _run(bigint, oracle, u, v, method)


def _addback_rows(seed, mu, mv, n, bits):
    """u = (qh v - 1) B^(mu - mv - 1) + low with v normalised: the quotient
    estimate from the top limbs is qh, one more than the true top limb, so the
    long division takes its add-back branch at the first quotient limb."""
    import random
    rng = random.Random(seed)
    U, V = [], []
    for _ in range(n):
        v = rng.getrandbits(bits * mv) | (1 << (bits * mv - 1))
        qh = rng.getrandbits(bits) | 1
        extra = mu - mv - 1
        u = ((qh * v - 1) << (bits * extra)) | rng.getrandbits(bits * extra) if extra else qh * v - 1
        U.append(u)
        V.append(v)
    return U, V


@pytest.mark.parametrize("method", ["auto", "shinv", "long"])
@pytest.mark.parametrize("bits", [64, 32])
@pytest.mark.parametrize("mu,mv", [(3, 2), (6, 5), (20, 16), (19, 18), (40, 31), (70, 64), (300, 200), (1500, 1024)])
def test_add_back_cases(bigint, oracle, bits, mu, mv, method):
    if bits == 32:
        mu, mv = 2 * mu, 2 * mv
    dtype = np.uint64 if bits == 64 else np.uint32
    U, V = _addback_rows(1000 + mu + mv, mu, mv, 4, bits)
    mask = (1 << bits) - 1
    u = np.array([[(x >> (bits * i)) & mask for i in range(mu)] for x in U], dtype)
    v = np.array([[(x >> (bits * i)) & mask for i in range(mv)] for x in V], dtype)
    B = bigint
    q, r, st = B.div(B.to_device(u), B.to_device(v), method=method)
    q, r = B.to_host(q, dtype), B.to_host(r, dtype)
    for i, (x, y) in enumerate(zip(U, V)):
        assert sum(int(w) << (bits * k) for k, w in enumerate(q[i])) == x // y
        assert sum(int(w) << (bits * k) for k, w in enumerate(r[i])) == x % y
    assert (st.cpu().numpy() == 0).all()


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


@pytest.mark.parametrize("mv,n", [(4, 1 << 20), (16, 1 << 18), (64, 1 << 16), (256, 1 << 14), (384, (1 << 23) // 768),
                                  (768, (1 << 23) // 1536), (1024, 1 << 12)])
def test_full_size_division_identity(bigint, mv, n):
    """The benchmark's division workloads at full size (2m/m limbs, u64),
    checked on every row by a property the division kernels do not share:
    q v has no limbs above 2m, u - q v = r with no borrow (so u = q v + r
    exactly), and r - v borrows (r < v) -- with the multiply and add/sub
    kernels."""
    import torch

    B = bigint
    from bigint_gb300.workloads import device_uniform_u64

    m2 = 2 * mv
    u = device_uniform_u64(11, n, m2)
    v = device_uniform_u64(12, n, mv)
    v[:, -1] |= 1
    q, r, st = B.div(u, v)
    assert (st == 0).all()
    vpad = torch.zeros((n, m2), dtype=torch.int64, device="cuda")
    vpad[:, :mv] = v
    qv = B.mulfull(q, vpad)                       # 4m limbs
    assert (qv[:, m2:] == 0).all()
    diff, borrow = B.sub(u, qv[:, :m2].contiguous())
    assert (borrow == 0).all()
    rpad = torch.zeros((n, m2), dtype=torch.int64, device="cuda")
    rpad[:, :mv] = r
    assert torch.equal(diff, rpad)
    _, lt = B.sub(r, v)
    assert (lt == 1).all()


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("mv,n", [(9, 40), (12, 3000), (16, 7000), (16, 9000), (12, 20000)])
def test_small_divisors_on_groups_and_threads(bigint, oracle, dtype, mv, n):
    """Divisors of 9..16 64-bit limbs: few instances run on 8-lane groups
    (div_small_on_groups), many on one thread each; both give the oracle's
    q and r, with add-backs forced on some rows (u = v * B^k - 1 style rows)."""
    w = 2 if dtype == np.uint32 else 1
    mu = 2 * mv * w
    u = uniform_limbs(301 + mv + n, n, mu, dtype)
    v = uniform_limbs(302 + mv + n, n, mv * w, dtype)
    v[:, -1] |= 1
    top = np.iinfo(dtype).max
    for i in range(0, n, 7):                       # v = B^k - 1 shaped divisors, u all ones
        v[i, :] = top
        u[i, :] = top
    _run(bigint, oracle, u, v, "auto")


@pytest.mark.parametrize("dtype", [np.uint64, np.uint32])
@pytest.mark.parametrize("method", ["auto", "long"])
@pytest.mark.parametrize("mv,n", [(20, 100), (32, 2000), (50, 300), (64, 2000), (100, 40), (128, 2000)])
def test_small_batches_on_warps_large_on_groups(bigint, oracle, mv, n, method, dtype):
    """Divisors of 17..128 64-bit limbs: up to 10 instances an SM divide on one
    warp each (div_small_on_warps), more on shared lane groups; the same (q, r)."""
    w = 2 if dtype == np.uint32 else 1           # u32 limbs a 64-bit limb
    u = uniform_limbs(311 + mv + n, n, 2 * mv * w, dtype)
    v = uniform_limbs(312 + mv + n, n, mv * w, dtype)
    v[:, -1] |= dtype(1)
    top = np.iinfo(dtype).max
    for i in range(0, n, 5):                       # all-ones rows: the estimate's q-hat = B - 1 branch
        v[i, :] = top
        u[i, :] = top
    _run(bigint, oracle, u, v, method)
