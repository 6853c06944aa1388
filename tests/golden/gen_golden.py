"""Generate the golden fixtures under tests/golden/.

Outputs are computed with Python's arbitrary-precision integers, which are
independent of both the oracle and the CUDA library.  Division cases are also
run through the reference's own prototypes/div.c (built by oracle/Makefile
into oracle/_ref/libref_div.so from the reference checkout) when it is
available, and the script refuses to write a fixture the reference
disagrees with.

The known-answer tests are the reference's own:
  * futhark/div.fut:185-186 -- u = [33986, 5952, 61904], v = [37752] in u16
    digits; the expected quotient [5764, 41927, 1] (u16) is stated there;
  * prototypes/Makefile:10 -- the fixed u32 vector `./div 0 8 ...`.

Usage:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "big-int_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from bigint_gb300.workloads import splitmix64  # noqa: E402


def to_int(limbs, bits):
    return sum(int(x) << (bits * i) for i, x in enumerate(limbs))


def from_int(x, m, bits):
    mask = (1 << bits) - 1
    return [(x >> (bits * i)) & mask for i in range(m)]


def rand_rows(seed, n, m, bits):
    raw = splitmix64(seed, n * m)
    if bits == 32:
        raw = raw & np.uint64(0xFFFFFFFF)
    return [[int(v) for v in raw[i * m:(i + 1) * m]] for i in range(n)]


def edge_rows(m, bits):
    top = (1 << bits) - 1
    return [
        ([0] * m, [0] * m),
        ([top] * m, [1] + [0] * (m - 1)),          # full-length carry / wrap
        ([top] * m, [top] * m),
        ([5] + [0] * (m - 1), [5] + [0] * (m - 1)),  # a == b
        ([0] * m, [1] + [0] * (m - 1)),            # a < b, borrow through all limbs
        ([0] * (m - 1) + [1], [1] + [0] * (m - 1)),
    ]


def gen_arith():
    cases = []
    seed = 7000
    for bits in (32, 64):
        for m in (1, 2, 3, 5, 8, 16, 33, 64):
            seed += 1
            rows_a = rand_rows(seed, 6, m, bits)
            rows_b = rand_rows(seed + 100000, 6, m, bits)
            pairs = list(zip(rows_a, rows_b)) + edge_rows(m, bits)
            a = [p[0] for p in pairs]
            b = [p[1] for p in pairs]
            add, sub, sign, mul, mulfull = [], [], [], [], []
            for x, y in pairs:
                X, Y = to_int(x, bits), to_int(y, bits)
                mod = 1 << (bits * m)
                add.append(from_int((X + Y) % mod, m, bits))
                sub.append(from_int(abs(X - Y), m, bits))
                sign.append(int(X < Y))
                mul.append(from_int((X * Y) % mod, m, bits))
                mulfull.append(from_int(X * Y, 2 * m, bits))
            cases.append(dict(bits=bits, m=m, a=a, b=b, add=add, sub=sub, sign=sign,
                              mul=mul, mulfull=mulfull))
    return cases


def gen_div(ref):
    cases = []
    seed = 9000
    for bits in (32, 64):
        for mu, mvs in ((2, (1, 2)), (3, (1, 2, 3)), (4, (2, 4)), (8, (1, 2, 3, 4, 8)),
                        (16, (1, 3, 8, 16)), (33, (2, 17, 33))):
            for mv in mvs:
                seed += 1
                n = 6
                u = rand_rows(seed, n, mu, bits)
                v = rand_rows(seed + 50000, n, mv, bits)
                # divisor precision sweep as prototypes/div.c:509-523 does
                for i in range(n):
                    nz = 1 + (i * mv) // n
                    v[i] = v[i][:nz] + [0] * (mv - nz)
                    if all(d == 0 for d in v[i]):
                        v[i][0] = 1
                q, r = [], []
                for x, y in zip(u, v):
                    X, Y = to_int(x, bits), to_int(y, bits)
                    q.append(from_int(X // Y, mu, bits))
                    r.append(from_int(X % Y, mv, bits))
                checked = False
                if ref is not None:
                    checked = check_with_reference(ref, u, v, q, r, bits, mu, mv)
                cases.append(dict(bits=bits, mu=mu, mv=mv, u=u, v=v, q=q, r=r,
                                  reference_div_checked=checked))
    return cases


def check_with_reference(ref, u, v, q, r, bits, mu, mv):
    """Run prototypes/div.c on the same inputs (u32 digit view, equal sizes)."""
    per = bits // 32
    M = mu * per
    U = np.zeros((len(u), M), np.uint32)
    V = np.zeros((len(u), M), np.uint32)
    for i, (x, y) in enumerate(zip(u, v)):
        U[i] = from_int(to_int(x, bits), M, 32)
        V[i] = from_int(to_int(y, bits), M, 32)
    qr, rr = ref(U, V)
    for i in range(len(u)):
        if to_int(qr[i], 32) != to_int(q[i], bits) or to_int(rr[i], 32) != to_int(r[i], bits):
            raise SystemExit(f"reference div.c disagrees with Python on case {i} (bits={bits}, mu={mu}, mv={mv})")
    return True


def gen_kat():
    kats = []
    # futhark/div.fut:185-186, u16 digits
    U16, V16, Q16 = [33986, 5952, 61904], [37752], [5764, 41927, 1]
    U, V, Q = to_int(U16, 16), to_int(V16, 16), to_int(Q16, 16)
    assert U // V == Q
    kats.append(dict(source="futhark/div.fut:185-186", bits=32, u=from_int(U, 2, 32),
                     v=from_int(V, 2, 32), q=from_int(Q, 2, 32), r=from_int(U % V, 2, 32)))
    # prototypes/Makefile:10
    u = [4254490950, 2896388618, 544147644, 1211343258, 1855778102, 4027074728, 1265731612, 2175660264]
    v = [2576532042, 4267266224, 725580630, 0, 0, 0, 0, 0]
    U, V = to_int(u, 32), to_int(v, 32)
    kats.append(dict(source="prototypes/Makefile:10", bits=32, u=u, v=v,
                     q=from_int(U // V, 8, 32), r=from_int(U % V, 8, 32)))
    return kats


def main():
    ref = None
    try:
        import oracle as O

        O.build()
        if O.ref_div_lib() is not None:
            ref = O.ref_div_u32
    except Exception as e:  # the fixtures do not depend on the reference being present
        print("reference div.c unavailable:", e)
    data = dict(
        generator="tests/golden/gen_golden.py",
        arith=gen_arith(),
        div=gen_div(ref),
        kat=gen_kat(),
    )
    if ref is not None:
        for k in data["kat"]:
            u = np.array([k["u"]], np.uint32)
            v = np.array([k["v"]], np.uint32)
            q, r = ref(u, v)
            assert [int(x) for x in q[0]] == k["q"] and [int(x) for x in r[0]] == k["r"], k["source"]
            k["reference_div_checked"] = True
    path = os.path.join(HERE, "golden.json")
    with open(path, "w") as f:
        json.dump(data, f, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes; reference div.c used:", ref is not None)


if __name__ == "__main__":
    main()
