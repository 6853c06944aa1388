"""GPU parity and behaviour of the serving loop (bi_server_*).

Every request of a mixed stream (add, sub, full multiply, division; sizes
log-uniform in 512..32768 bits; operands in one device-resident pool) is
compared with the oracle; each result is the same in the mix (Poisson
arrivals, and a burst where every request is in flight at once), alone (one
request at a time through the server) and through the plain per-request
launches; admission under a small result arena and a small ring (BI_EBUSY
back-pressure) keeps every result; the loop leaves when idle and is
relaunched; invalid requests are rejected on the host.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POOL = 1 << 20


def _W():
    from bigint_gb300 import workloads as W

    return W


@pytest.fixture(scope="module")
def setup(bigint):
    import torch

    W = _W()
    d, arrival, pool_seed = W.serve_stream(600, 200_000, seed=77, pool_limbs=POOL)
    pool = W.serve_pool_device(POOL, pool_seed)
    host = W.splitmix64(pool_seed, POOL)
    # a stripe of all-ones limbs and one of zeros for carry chains and zero divisors
    host[1024:3072] = np.uint64(0xFFFFFFFFFFFFFFFF)
    host[4096:6144] = 0
    pool.copy_(torch.from_numpy(host.view(np.int64)).cuda())
    torch.cuda.synchronize()
    return d, arrival, pool, host


def _arena(limbs):
    import torch

    return torch.zeros(limbs, dtype=torch.int64, device="cuda")


def _out_limbs(d):
    B = __import__("bigint_gb300")
    m = d["m"].astype(np.int64)
    rl = np.where(d["op"] == B.OP_MULFULL, 2 * m, np.where(d["op"] == B.OP_DIV, m + d["mb"], m))
    return int(((rl + 1) // 2 * 2).sum())


def _collect(B, d, comp, arena_host):
    """Per request: (result limbs, remainder limbs or None, status)."""
    res = []
    for i in range(len(d)):
        op, m, mb = int(d["op"][i]), int(d["m"][i]), int(d["mb"][i])
        r = int(comp["r"][i])
        if op == B.OP_MULFULL:
            res.append((arena_host[r: r + 2 * m].copy(), None, int(comp["status"][i])))
        elif op == B.OP_DIV:
            r2 = int(comp["r2"][i])
            res.append((arena_host[r: r + m].copy(), arena_host[r2: r2 + mb].copy(), int(comp["status"][i])))
        else:
            res.append((arena_host[r: r + m].copy(), None, int(comp["status"][i])))
    return res


def _check_oracle(B, oracle, d, host, res):
    for i in range(len(d)):
        op, m, mb = int(d["op"][i]), int(d["m"][i]), int(d["mb"][i])
        a = host[int(d["a"][i]): int(d["a"][i]) + m][None, :]
        b = host[int(d["b"][i]): int(d["b"][i]) + mb][None, :]
        got, got2, st = res[i]
        if op == B.OP_ADD:
            assert (got == oracle.add(a, b)[0]).all(), ("add", i, m)
        elif op == B.OP_SUB:
            r, s = oracle.sub(a, b)
            assert (got == r[0]).all() and st == int(s[0]), ("sub", i, m)
        elif op == B.OP_MULFULL:
            assert (got == oracle.mulfull(a, b)[0]).all(), ("mulfull", i, m)
        elif op == B.OP_MUL:
            assert (got == oracle.mul(a, b)[0]).all(), ("mul", i, m)
        else:
            q, r, s = oracle.div(a, b)
            assert (got == q[0]).all() and (got2 == r[0]).all() and st == int(s[0]), ("div", i, m, mb)


def _same(x, y):
    assert len(x) == len(y)
    for i, (p, q) in enumerate(zip(x, y)):
        assert (p[0] == q[0]).all(), i
        assert (p[1] is None) == (q[1] is None) and (p[1] is None or (p[1] == q[1]).all()), i
        assert p[2] == q[2], i


def _host(t):
    return t.cpu().numpy().view(np.uint64)


def _run_alone(B, srv, d):
    """Each request on its own: submit, wait for its completion, copy it out."""
    arena = srv.arena
    out = []
    for i in range(len(d)):
        t = srv.submit(d[i])
        assert t is not None
        deadline = time.time() + 10
        c = srv.poll(4)
        while len(c) == 0:
            assert time.time() < deadline, "request did not complete"
            c = srv.poll(4)
        assert len(c) == 1 and int(c["ticket"][0]) == t
        comp = np.zeros(1, dtype=B.COMPLETION_DTYPE)
        comp[0] = c[0]
        out.append(_collect(B, d[i: i + 1], comp, _host(arena))[0])
        srv.release(t)
    return out


@pytest.fixture(scope="module")
def mix_results(bigint, setup):
    """The Poisson stream through the server (all results kept in the arena)."""
    B = bigint
    d, arrival, pool, host = setup
    arena = _arena(_out_limbs(d) + 16)
    with B.Server(pool, arena) as srv:
        lat, comp, rep = srv.replay(d, arrival)
    assert rep["requests"] == len(d)
    assert (lat > 0).all()
    return _collect(B, d, comp, _host(arena)), rep


def test_mixed_stream_matches_oracle(bigint, oracle, setup, mix_results):
    d, _, _, host = setup
    res, rep = mix_results
    _check_oracle(bigint, oracle, d, host, res)
    assert rep["p99_us"] >= rep["p50_us"] > 0


def test_burst_overlaps_and_matches_mix(bigint, setup, mix_results):
    """All requests submitted at once: they complete out of submission order
    (small ones overtake large ones on the device) with the same results."""
    B = bigint
    d, _, pool, _ = setup
    arena = _arena(_out_limbs(d) + 16)
    with B.Server(pool, arena) as srv:
        tickets = [srv.submit(d[i]) for i in range(len(d))]
        assert None not in tickets
        order = []
        comp = np.zeros(len(d), dtype=B.COMPLETION_DTYPE)
        deadline = time.time() + 30
        while len(order) < len(d):
            assert time.time() < deadline
            for c in srv.poll():
                k = int(c["ticket"]) - tickets[0]
                comp[k] = c
                order.append(k)
        assert sorted(order) == list(range(len(d)))
        assert order != sorted(order), "no request overtook another"
        res = _collect(B, d, comp, _host(arena))
        for k in range(len(d)):
            srv.release(tickets[k])
    _same(res, mix_results[0])


def test_alone_equals_mix(bigint, setup, mix_results):
    B = bigint
    d, _, pool, _ = setup
    with B.Server(pool, _arena(8192)) as srv:
        alone = _run_alone(B, srv, d)
    _same(alone, mix_results[0])


def test_plain_launch_equals_mix(bigint, setup, mix_results):
    B = bigint
    d, arrival, pool, _ = setup
    arena = _arena(_out_limbs(d) + 16)
    lat, comp, rep = B.replay_plain(pool, arena, d, arrival, streams=4)
    assert rep["launches"] == len(d)
    _same(_collect(B, d, comp, _host(arena)), mix_results[0])


def test_backpressure_small_arena_and_ring(bigint, setup, mix_results):
    """Arena of 4096 limbs and 8 ring slots: submissions are refused
    (BI_EBUSY) until earlier results are released; every result still
    matches the mix."""
    B = bigint
    d, _, pool, _ = setup
    n = 200
    arena = _arena(4096)
    got = [None] * n
    busy = 0
    with B.Server(pool, arena, ring_slots=8) as srv:
        nxt, tick = 0, {}
        deadline = time.time() + 60
        while any(g is None for g in got):
            assert time.time() < deadline
            while nxt < n:
                t = srv.submit(d[nxt])
                if t is None:
                    busy += 1
                    break
                tick[t] = nxt
                nxt += 1
            cs = srv.poll()
            if len(cs):
                host_arena = _host(arena)
                for c in cs:
                    i = tick[int(c["ticket"])]
                    comp = np.zeros(1, dtype=B.COMPLETION_DTYPE)
                    comp[0] = c
                    got[i] = _collect(B, d[i: i + 1], comp, host_arena)[0]
                    srv.release(int(c["ticket"]))
        assert srv.info()["busy"] >= busy > 0
    _same(got, mix_results[0][:n])


def test_idle_exit_and_relaunch(bigint, setup):
    B = bigint
    d, _, pool, _ = setup
    with B.Server(pool, _arena(8192), idle_us=200) as srv:
        first = _run_alone(B, srv, d[:3])
        time.sleep(0.05)   # far past the idle limit: every CTA has left
        second = _run_alone(B, srv, d[:3])
        assert srv.info()["launches"] >= 2
    _same(first, second)


def test_edge_requests(bigint, oracle, setup):
    """Carry chains through all-ones limbs, a zero divisor (status 1, zero
    quotient and remainder), m = 1, the largest size, odd offsets."""
    B = bigint
    _, _, pool, host = setup
    reqs = [
        (B.OP_ADD, 512, 512, 1024, 1024),       # ones + ones
        (B.OP_SUB, 300, 300, 1024, 1500),       # equal operands: zero, sign 0
        (B.OP_SUB, 64, 64, 4096, 1024),         # 0 - ones: sign 1
        (B.OP_MULFULL, 512, 512, 1024, 2048),   # ones * ones
        (B.OP_DIV, 512, 256, 1024, 4096),       # divisor zero
        (B.OP_DIV, 512, 256, 1024, 2048),       # ones / ones
        (B.OP_DIV, 7, 7, 1025, 9001),           # equal sizes, odd offsets
        (B.OP_ADD, 1, 1, 7, 9),                 # single limb, odd offsets
        (B.OP_SUB, 33, 33, 11, 13),
        (B.OP_MUL, 100, 100, 3, 5),             # truncated product
        (B.OP_MULFULL, 1, 1, 1, 3),
        (B.OP_DIV, 512, 1, 20000, 40001),       # one-limb divisor
    ]
    d = np.zeros(len(reqs), dtype=B.DESC_DTYPE)
    for i, (op, m, mb, a, b) in enumerate(reqs):
        d[i]["op"], d[i]["m"], d[i]["mb"], d[i]["a"], d[i]["b"] = op, m, mb, a, b
    with B.Server(pool, _arena(8192)) as srv:
        res = _run_alone(B, srv, d)
    _check_oracle(B, oracle, d, host, res)
    assert res[4][2] == 1 and not res[4][0].any() and not res[4][1].any()
    assert res[1][2] == 0 and not res[1][0].any()
    assert res[2][2] == 1


def test_invalid_requests_rejected(bigint, setup):
    B = bigint
    _, _, pool, _ = setup
    with B.Server(pool, _arena(4096), max_limbs=256) as srv:
        def bad(op, m, mb, a, b):
            d = np.zeros(1, dtype=B.DESC_DTYPE)
            d[0]["op"], d[0]["m"], d[0]["mb"], d[0]["a"], d[0]["b"] = op, m, mb, a, b
            with pytest.raises(B.BigIntError):
                srv.submit(d[0])

        bad(9, 8, 8, 0, 0)                        # unknown op
        bad(B.OP_ADD, 0, 0, 0, 0)                 # m = 0
        bad(B.OP_ADD, 257, 257, 0, 0)             # above max_limbs
        bad(B.OP_DIV, 8, 9, 0, 0)                 # divisor longer than dividend
        bad(B.OP_DIV, 8, 0, 0, 0)                 # empty divisor
        bad(B.OP_MULFULL, 8, 8, POOL - 4, 0)      # operand past the pool
        with pytest.raises(B.BigIntError):
            srv.release(0)                        # nothing in flight
        assert srv.info()["submitted"] == 0


def test_destroy_with_requests_in_flight(bigint, setup):
    """Destroying a server with queued requests lets them finish and returns."""
    B = bigint
    d, _, pool, _ = setup
    srv = B.Server(pool, _arena(_out_limbs(d) + 16))
    for i in range(len(d)):
        assert srv.submit(d[i]) is not None
    srv.close()
    with B.Server(pool, _arena(8192)) as srv2:   # the device is usable again
        _run_alone(B, srv2, d[:2])


def test_dropped_request_times_out_and_the_loop_goes_on(bigint, oracle, setup):
    """Failure injection on the host: a published slot whose contents never
    arrive.  The claiming CTA's bounded wait gives up after a second and
    completes that request with status 255; requests around it complete
    normally, during the wait, with the right results."""
    B = bigint
    d, _, pool, host = setup
    with B.Server(pool, _arena(8192), idle_us=3_000_000) as srv:
        t0 = srv.submit(d[0])
        tl = srv.inject_dropped()
        t1 = srv.submit(d[1])
        done = {}
        deadline = time.time() + 20
        while len(done) < 3:
            assert time.time() < deadline, "no completion for the dropped request"
            for c in srv.poll():
                done[int(c["ticket"])] = c
        assert int(done[tl]["status"]) == 255
        assert srv.info()["lost"] == 1
        arena = _host(srv.arena)
        for t, i in ((t0, 0), (t1, 1)):
            comp = np.zeros(1, dtype=B.COMPLETION_DTYPE)
            comp[0] = done[t]
            res = _collect(B, d[i: i + 1], comp, arena)
            _check_oracle(B, oracle, d[i: i + 1], host, res)
        for t in (t0, tl, t1):
            srv.release(t)


def _word_requests(B, d, n=300):
    """The stream's first n requests as 32-bit-word requests (width 32): odd
    and even word counts, some at odd word offsets of the same pool."""
    w = d[:n].copy()
    for i in range(n):
        m, mb = int(w["m"][i]), int(w["mb"][i])
        mw = 2 * m - (i & 1)
        mbw = min(mw, 2 * mb - ((i >> 1) & 1)) if int(w["op"][i]) == B.OP_DIV else mw
        w[i]["m"], w[i]["mb"], w[i]["width"] = mw, mbw, 32
        w[i]["a"] = 2 * int(w["a"][i]) + (1 if i % 3 == 0 else 0)
        w[i]["b"] = 2 * int(w["b"][i]) + (1 if i % 5 == 0 else 0)
    return w


def _word_arena_limbs(B, d):
    m = d["m"].astype(np.int64)
    e = np.where(d["op"] == B.OP_MULFULL, 2 * m, np.where(d["op"] == B.OP_DIV, m + d["mb"], m))
    limbs = (e + 1) // 2
    return int(((limbs + 1) // 2 * 2).sum())


def test_word_requests_match_oracle_and_plain(bigint, oracle, setup):
    """32-bit-word requests (the reference's U32bits layout) through the
    loop: results at word offsets equal the oracle's on the words and the
    plain per-request launches' (bi_*_u32)."""
    B = bigint
    d, arrival, pool, host = setup
    w = _word_requests(B, d)
    h32 = host.view(np.uint32)
    arena = _arena(_word_arena_limbs(B, w) + 16)
    with B.Server(pool, arena) as srv:
        lat, comp, rep = srv.replay(w, arrival[: len(w)])
    assert rep["requests"] == len(w)
    res = _collect(B, w, comp, _host(arena).view(np.uint32))
    _check_oracle(B, oracle, w, h32, res)
    arena2 = _arena(_word_arena_limbs(B, w) + 16)
    _, comp2, _ = B.replay_plain(pool, arena2, w, arrival[: len(w)], streams=2)
    _same(res, _collect(B, w, comp2, _host(arena2).view(np.uint32)))


def test_word_request_checks(bigint, setup):
    """A word request is checked in words: an operand past the pool's
    2 x limbs words and a width other than 0, 32 or 64 are refused."""
    B = bigint
    d, _, pool, _ = setup
    with B.Server(pool, _arena(1 << 16)) as srv:
        bad = d[:1].copy()
        bad[0]["width"], bad[0]["op"], bad[0]["m"] = 32, B.OP_ADD, 8
        bad[0]["a"] = 2 * POOL - 7
        with pytest.raises(B.BigIntError):
            srv.submit(bad[0])
        bad[0]["a"], bad[0]["width"] = 0, 16
        with pytest.raises(B.BigIntError):
            srv.submit(bad[0])
