"""CPU model of block long division (big-int_gb300/csrc/divblock.cuh), lane
by lane on Python integers, checked against exact division.

The model follows the kernel's steps with the kernel's index arithmetic:
the divisor right-aligned in NL lanes of VPL limbs (MX = NL VPL positions),
the window of MX + KB limbs (the top lane's X[VPL ..] holding the KB limbs
above the divisor), the padded first block, per block the small long division
of the top 2 KB + 1 window limbs by the divisor's top KB + 1 limbs (capped at
B^KB - 1, its remainder left in place), every lane's KB rows with the part
above its limbs added to its spill, the spill subtracted by the next lane
with its rare borrow run on through the lane, the lane-to-lane borrows, the
sign of the limb above the divisor deciding the add-back, the quotient
limbs stored, the window moved up KB limbs with KB dividend limbs entering at
the bottom, and the remainder read back shifted right.  Small shapes (2 to 4
lanes of 5 to 16 limbs) reach every branch -- capped block estimates, add-backs,
spill borrows -- on random and constructed inputs.  It is a model of the
algorithm, not of the GPU: the GPU tests compare the kernel with the oracle.
"""
import random

M = (1 << 64) - 1
B = 1 << 64


def _int(limbs):
    return sum(x << (64 * k) for k, x in enumerate(limbs))


def div_blk_model(u, v, VPL, KB, NL, stats):
    MU, MV = len(u), len(v)
    MX = NL * VPL
    assert MV <= MX and VPL >= KB + 1 and 32 % KB == 0
    K = max((i + 1 for i in range(MV) if v[i]), default=0)
    if K == 0:
        return [0] * MU, [0] * MV, 1
    if MU < K:
        return [0] * MU, [u[i] if i < MU else 0 for i in range(MV)], 0
    s = 64 - v[K - 1].bit_length()
    zl = MX - K

    def vl(j):
        return v[j] if 0 <= j < K else 0

    def raw(t):
        return u[t] if 0 <= t < MU else 0

    def sh(t):
        return ((raw(t) << s) & M) | ((raw(t - 1) >> 1) >> (63 - s))

    D = [[((vl(gl * VPL + i - zl) << s) & M) | ((vl(gl * VPL + i - zl - 1) >> 1) >> (63 - s)) for i in range(VPL)]
         for gl in range(NL)]
    top = NL - 1
    nq = MU - K + 1
    pad = (KB - nq % KB) % KB
    nblk = (nq + pad) // KB
    x0 = MU + pad - MX - KB + 1
    X = [[sh(x0 + gl * VPL + i) for i in range(VPL)] + [0] * KB for gl in range(NL)]
    for i in range(KB):
        X[top][VPL + i] = sh(x0 + MX + i)
    q = [0] * MU
    Vp = _int(D[top][VPL - KB - 1:VPL])
    for b in range(nblk):
        # the block's quotient from the top 2 KB + 1 window limbs, in place
        U = _int(X[top][VPL - KB - 1:VPL + KB])
        if U >> (64 * KB) >= Vp:
            stats["cap"] += 1
            Q = B ** KB - 1
        else:
            Q = U // Vp
        U -= Q * Vp
        assert 0 <= U < 2 * B ** (KB + 1)
        X[top][VPL - KB - 1:VPL + KB] = [(U >> (64 * k)) & M for k in range(2 * KB + 1)]
        t0 = X[top][VPL]
        Qb = [(Q >> (64 * k)) & M for k in range(KB)]
        # rows: X -= Qb x D (the top lane without its top KB + 1 limbs), spill S
        spills = []
        for gl in range(NL):
            Dm = [0 if (gl == top and c >= VPL - KB - 1) else D[gl][c] for c in range(VPL)]
            Xl, S = X[gl], [0] * (KB + 1)
            for I in range(KB):
                for part, shift in ((0, 0), (1, 1)):     # low halves at I + c, high halves at I + c + 1
                    br = 0
                    for c in range(VPL - I - shift):
                        y = (Qb[I] * Dm[c]) >> (64 * part) & M
                        t = Xl[I + shift + c] - y - br
                        br, Xl[I + shift + c] = (1 if t < 0 else 0), t & M
                    cy = br
                    for c in range(I + shift):
                        y = (Qb[I] * Dm[VPL - I - shift + c]) >> (64 * part) & M
                        t = S[c] + y + cy
                        cy, S[c] = t >> 64, t & M
                    S[I + shift] += cy
                    assert S[I + shift] <= M
            spills.append(S)
        assert all(x == 0 for x in spills[top][1:])     # the top lane spills borrows only
        tv = t0 - spills[top][0]
        # the spill of the lane below; generate / propagate
        g, p = [0] * NL, [0] * NL
        for gl in range(NL):
            Sin = spills[gl - 1] if gl else [0] * (KB + 1)
            Xl, br = X[gl], 0
            for k in range(KB + 1):
                t = Xl[k] - Sin[k] - br
                br, Xl[k] = (1 if t < 0 else 0), t & M
            if br:
                stats["spill_borrow"] += 1
                for i in range(KB + 1, VPL):
                    y = Xl[i]
                    Xl[i] = (y - br) & M
                    br = br if y == 0 else 0
            g[gl], p[gl] = br, int(all(x == 0 for x in Xl[:VPL]))
        c = 0
        for gl in range(NL):
            bin_ = c
            c = g[gl] | (p[gl] & c)
            for i in range(VPL):
                if not bin_:
                    break
                y = X[gl][i]
                X[gl][i] = (y - 1) & M
                bin_ = 1 if y == 0 else 0
        assert tv - c in (0, -1)
        if tv != c:                                        # one too large: add D back
            stats["add_back"] += 1
            Q -= 1
            Qb = [(Q >> (64 * k)) & M for k in range(KB)]
            cy = 0
            for gl in range(NL):
                for i in range(VPL):
                    t = X[gl][i] + D[gl][i] + cy
                    cy, X[gl][i] = t >> 64, t & M
            assert cy == 1
        qb = nq + pad - (b + 1) * KB
        for k in range(KB):
            if qb + k < nq:
                q[qb + k] = Qb[k]
            else:
                assert Qb[k] == 0                          # the first block's pad limbs
        if b + 1 < nblk:                                   # move up KB limbs; KB dividend limbs enter
            old = [row[:] for row in X]
            for gl in range(NL):
                for i in range(VPL + KB - 1, KB - 1, -1):
                    X[gl][i] = old[gl][i - KB]
                for i in range(KB):
                    X[gl][i] = old[gl - 1][VPL - KB + i] if gl else sh(x0 - (b + 1) * KB + i)

    def pos(pp):
        return 0 if pp >= MX else X[pp // VPL][pp % VPL]

    r = [0] * MV
    for j in range(K):
        pp = zl + j
        r[j] = (pos(pp) >> s) | ((pos(pp + 1) << 1) << (63 - s)) & M
    return q, r, 0


def _check(u, v, shape, stats):
    q, r, st = div_blk_model(u, v, *shape, stats)
    U, V = _int(u), _int(v)
    if V == 0:
        assert st == 1 and not any(q) and not any(r)
        return
    assert (_int(q), _int(r)) == divmod(U, V), (len(u), len(v), shape)


SHAPES = [(5, 4, 2), (9, 8, 2), (16, 8, 2), (8, 4, 4), (16, 8, 1)]   # (VPL, KB, lanes)


def test_random_and_edge_inputs():
    rng = random.Random(5)
    stats = {"cap": 0, "add_back": 0, "spill_borrow": 0}
    for VPL, KB, NL in SHAPES:
        MX = VPL * NL
        for _ in range(60):
            mv = rng.randint(1, MX)
            mu = rng.randint(mv, 3 * MX)
            for kind in ("rand", "short", "ones", "pow", "near"):
                u = [rng.getrandbits(64) for _ in range(mu)]
                v = [rng.getrandbits(64) for _ in range(mv)]
                if kind == "short":
                    k = rng.randint(1, mv)
                    v = v[:k - 1] + [v[k - 1] | 1] + [0] * (mv - k)
                elif kind == "ones":
                    u, v = [M] * mu, [M] * mv
                elif kind == "pow":
                    v = [0] * mv
                    v[rng.randrange(mv)] = 1 << rng.randrange(64)
                elif kind == "near" and mu > mv:           # u = Q v + v - 1: every estimate on its edge
                    v[-1] |= 1 << 63
                    Ui = rng.getrandbits(64 * (mu - mv)) * _int(v) + _int(v) - 1
                    Ui = min(Ui, B ** mu - 1)
                    u = [(Ui >> (64 * k)) & M for k in range(mu)]
                _check(u, v, (VPL, KB, NL), stats)
    assert stats["add_back"] > 20 and stats["spill_borrow"] > 20


def test_capped_block_estimates():
    """u = v B^(mu - mv) - 1 with divisors whose top limbs sit just above a
    power of two: the block estimate from the truncated operands reaches B^KB
    and is capped at B^KB - 1."""
    rng = random.Random(9)
    stats = {"cap": 0, "add_back": 0, "spill_borrow": 0}
    for VPL, KB, NL in SHAPES:
        MX = VPL * NL
        for mv in sorted({KB + 1, KB + 2, MX // 2, MX}):
            for mu in (mv + 1, mv + KB, 2 * mv, 3 * mv + 1):
                for variant in range(3):
                    if variant == 0:
                        v = [M] * (mv - 1) + [1 << 63]
                    elif variant == 1:
                        v = [M] * (mv - 1) + [(1 << 63) | (M >> 1)]
                    else:
                        v = ([rng.getrandbits(64) | (1 << 63) for _ in range(max(0, mv - KB - 2))] + [M] * (KB + 2))[-mv:]
                    Ui = _int(v) * B ** (mu - mv) - 1
                    _check([(Ui >> (64 * k)) & M for k in range(mu)], v, (VPL, KB, NL), stats)
    assert stats["cap"] > 100
