"""CPU tests: the oracle against the golden fixtures, the reference's KATs,
Python integers, and (where it was built) the reference's own div.c."""
import numpy as np
import pytest

from conftest import limbs
from bigint_gb300.workloads import splitmix64


def _int(row):
    bits = row.dtype.itemsize * 8
    return sum(int(x) << (bits * i) for i, x in enumerate(row))


def test_little_endian(oracle):
    assert oracle.lib().orc_little_endian() == 1


def test_golden_arith(oracle, golden):
    for c in golden["arith"]:
        a, b = limbs(c["a"], c["bits"]), limbs(c["b"], c["bits"])
        assert (oracle.add(a, b) == limbs(c["add"], c["bits"])).all()
        r, s = oracle.sub(a, b)
        assert (r == limbs(c["sub"], c["bits"])).all()
        assert (s == np.array(c["sign"], np.uint8)).all()
        assert (oracle.mul(a, b) == limbs(c["mul"], c["bits"])).all()
        assert (oracle.mulfull(a, b) == limbs(c["mulfull"], c["bits"])).all()


def test_golden_div(oracle, golden):
    for c in golden["div"]:
        u, v = limbs(c["u"], c["bits"]), limbs(c["v"], c["bits"])
        q, r, st = oracle.div(u, v)
        assert (st == 0).all()
        assert (q == limbs(c["q"], c["bits"])).all(), (c["bits"], c["mu"], c["mv"])
        assert (r == limbs(c["r"], c["bits"])).all(), (c["bits"], c["mu"], c["mv"])


def test_reference_kats(oracle, golden):
    for k in golden["kat"]:
        u, v = limbs([k["u"]], 32), limbs([k["v"]], 32)
        q, r, _ = oracle.div(u, v)
        assert [int(x) for x in q[0]] == k["q"], k["source"]
        assert [int(x) for x in r[0]] == k["r"], k["source"]


def test_kat_values_stated_by_reference():
    # futhark/div.fut:185-186 states the u16 quotient [5764, 41927, 1]
    U = 33986 + (5952 << 16) + (61904 << 32)
    assert U // 37752 == 5764 + (41927 << 16) + (1 << 32)


@pytest.mark.parametrize("m", [2, 5, 16, 40])
def test_div_matches_reference_div_c(oracle, m):
    if oracle.ref_div_lib() is None:
        pytest.skip("reference div.c not built here")
    n = 3 * m
    u = (splitmix64(11 + m, n * m) & np.uint64(0xFFFFFFFF)).astype(np.uint32).reshape(n, m)
    v = (splitmix64(12 + m, n * m) & np.uint64(0xFFFFFFFF)).astype(np.uint32).reshape(n, m)
    for i in range(n):                      # divisor precisions 1..m (div.c:509-523)
        v[i, 1 + i % m:] = 0
        v[i, 0] |= 1
    q, r, _ = oracle.div(u, v)
    qr, rr = oracle.ref_div_u32(u, v)
    assert (q == qr).all() and (r == rr).all()


def test_div_special_cases(oracle):
    B = 1 << 32
    cases = [
        (B**4 - 1, 1), (B**4 - 1, B - 1), (B**3, B), (B**3, B**2), (B**3 + 5, B**2),
        (B**4 - 1, B**3 + 1), (12345, 1 << 100), (B**4 - 1, (B**4 - 1) // 2 + 1),
        (0, 7), (B**4 - 2, B**4 - 1), (B**4 - 1, B**4 - 1), (B**2 * 3, 2 * B + 1),
    ]
    m = 5
    u = np.array([[(x >> (32 * i)) & (B - 1) for i in range(m)] for x, _ in cases], np.uint32)
    v = np.array([[(y >> (32 * i)) & (B - 1) for i in range(m)] for _, y in cases], np.uint32)
    q, r, _ = oracle.div(u, v)
    for i, (x, y) in enumerate(cases):
        assert _int(q[i]) == x // y and _int(r[i]) == x % y, (x, y)


def test_div_by_zero_flagged(oracle):
    u = np.ones((2, 4), np.uint64)
    v = np.zeros((2, 2), np.uint64)
    v[1, 0] = 3
    q, r, st = oracle.div(u, v)
    assert list(st) == [1, 0]
    assert (q[0] == 0).all() and (r[0] == 0).all()


def test_threaded_matches_single(oracle):
    n, m = 64, 12
    a = splitmix64(5, n * m).reshape(n, m)
    b = splitmix64(6, n * m).reshape(n, m)
    assert (oracle.mulfull(a, b, nthreads=4) == oracle.mulfull(a, b)).all()
    r1, s1 = oracle.sub(a, b, nthreads=3)
    r2, s2 = oracle.sub(a, b)
    assert (r1 == r2).all() and (s1 == s2).all()


# A documented defect of the reference's division prototype: its single
# delta step (prototypes/div.c:459-463) leaves q one short for some inputs.
REF_DIV_DEFECT = (0xdc4461359674c9cfd718dc1b567834b5, 0xdd2982a538271953, 4)


def _digits(x, m):
    return [(x >> (32 * i)) & 0xFFFFFFFF for i in range(m)]


def test_faithful_restatement_matches_reference_div_c(oracle):
    """div_ref is div.c as written: identical outputs, defect included."""
    if oracle.ref_div_lib() is None:
        pytest.skip("reference div.c not built here")
    for m in (3, 4, 5, 8, 16):
        n = 600
        u = (splitmix64(40 + m, n * m) & np.uint64(0xFFFFFFFF)).astype(np.uint32).reshape(n, m)
        v = (splitmix64(41 + m, n * m) & np.uint64(0xFFFFFFFF)).astype(np.uint32).reshape(n, m)
        for i in range(n):
            v[i, 1 + i % m:] = 0
            v[i, 0] |= 1
        q1, r1, _ = oracle.div_ref(u, v)
        q2, r2 = oracle.ref_div_u32(u, v)
        assert (q1 == q2).all() and (r1 == r2).all()


def test_reference_division_defect_and_exact_oracle(oracle):
    U, V, m = REF_DIV_DEFECT
    u = np.array([_digits(U, m)], np.uint32)
    v = np.array([_digits(V, m)], np.uint32)
    qf, rf, _ = oracle.div_ref(u, v)
    assert _int(qf[0]) == U // V - 1 and _int(rf[0]) == U % V + V     # r >= v: not reduced
    if oracle.ref_div_lib() is not None:
        qr, rr = oracle.ref_div_u32(u, v)
        assert _int(qr[0]) == U // V - 1
    q, r, _ = oracle.div(u, v)
    assert _int(q[0]) == U // V and _int(r[0]) == U % V


def test_exact_oracle_division_random(oracle):
    for m in (4, 5, 6, 8):
        n = 1500
        u = (splitmix64(70 + m, n * m) & np.uint64(0xFFFFFFFF)).astype(np.uint32).reshape(n, m)
        v = (splitmix64(71 + m, n * m) & np.uint64(0xFFFFFFFF)).astype(np.uint32).reshape(n, m)
        nz = 1 + np.arange(n) % m
        for i in range(n):
            v[i, nz[i]:] = 0
            v[i, nz[i] - 1] |= 1
        q, r, _ = oracle.div(u, v)
        for i in range(n):
            U, V = _int(u[i]), _int(v[i])
            assert _int(q[i]) == U // V and _int(r[i]) == U % V


def test_primitive_restatements_against_python_ints(oracle):
    """The oracle's restatements of div.c's helpers against Python integers."""
    from bigint_gb300.workloads import uniform_limbs

    O = oracle
    for dtype, bits in ((np.uint64, 64), (np.uint32, 32)):
        a = uniform_limbs(71, 40, 9, dtype)
        b = a.copy()
        b[::3, 4] ^= dtype(1)
        a[5] = 0
        a[6, 3:] = 0
        ints_a = [O.to_int(r) for r in a]
        ints_b = [O.to_int(r) for r in b]
        assert list(O.cmp_rows(a, b)) == [(x > y) - (x < y) for x, y in zip(ints_a, ints_b)]
        k, z = O.findk_rows(a)
        assert list(z) == [1 if x == 0 else 0 for x in ints_a]
        assert list(k) == [max(0, (x.bit_length() - 1) // bits) for x in ints_a]
        for sh in (-3, 0, 2, 9):
            r = O.shift_rows(a, sh)
            want = [(x << (bits * sh)) % (1 << (bits * 9)) if sh >= 0 else x >> (bits * -sh) for x in ints_a]
            assert [O.to_int(row) for row in r] == want
        d = uniform_limbs(72, 40, 1, dtype)[:, 0]
        d[0] = 0
        d[1] = 1
        d[2] = np.iinfo(dtype).max
        assert [O.to_int(r) for r in O.muld_rows(a, d)] == [(x * int(dd)) % (1 << (bits * 9)) for x, dd in zip(ints_a, d)]
        q, rem = O.quod_rows(a, d)
        for x, dd, qq, rr in zip(ints_a, d, q, rem):
            dd = int(dd)
            assert O.to_int(qq) == (x // dd if dd else 0) and int(rr) == (x % dd if dd else 0)


def test_division_word_products_count(oracle):
    """orc_div_ref_word_products_u32 counts the reference division's
    multiplications on significant digits: zero for a zero divisor; for a
    one-digit divisor the inverse is a digit division (no product), so the
    count is sig(u) * sig(floor(B^h / v)) + sig(q) exactly; and it grows
    with the size."""
    B = 1 << 32
    assert oracle.div_ref_word_products(np.arange(1, 9, dtype=np.uint32), np.zeros(8, np.uint32)) == 0
    rng = np.random.default_rng(7)
    for m in (4, 9, 16):
        u = rng.integers(1, 2**32, size=m, dtype=np.uint32)
        v0 = int(rng.integers(2, 2**32))
        h = m
        w = (B ** h) // v0
        q = _int(u) // v0
        sig = lambda x: (x.bit_length() + 31) // 32
        want = h * sig(w) + sig(q)
        got = oracle.div_ref_word_products(u, np.array([v0], np.uint32))
        assert got == want, (m, got, want)
    wp = []
    for m in (8, 32, 128):
        u = rng.integers(0, 2**32, size=2 * m, dtype=np.uint32)
        v = rng.integers(0, 2**32, size=m, dtype=np.uint32)
        v[-1] |= 1
        wp.append(oracle.div_ref_word_products(u, v))
    assert wp[0] < wp[1] < wp[2] and wp[2] > 16 * wp[0]
