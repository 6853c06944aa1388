"""GPU parity of the uneven-batch plan (bi_plan_*): every instance of a mixed
batch of add, sub, full multiply and division over sizes log-uniform in
256..8192 bits is compared with the oracle; large instances of each
operation; graph replay, recapture on new arenas and autotuning leave the
results unchanged; invalid descriptors are rejected."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _groups(d):
    keys = {}
    for i, (op, m, mb) in enumerate(zip(d["op"], d["m"], d["mb"])):
        keys.setdefault((int(op), int(m), int(mb)), []).append(i)
    return keys


def check_batch(B, oracle, d, arena, out, flags, nthreads=1):
    """Compare every instance of the batch with the oracle, grouped by shape."""
    for (op, m, mb), idx in _groups(d).items():
        idx = np.array(idx)
        a = np.stack([arena[d["a"][i]: d["a"][i] + m] for i in idx])
        b = np.stack([arena[d["b"][i]: d["b"][i] + mb] for i in idx])
        if op == B.OP_ADD:
            got = np.stack([out[d["r"][i]: d["r"][i] + m] for i in idx])
            assert (got == oracle.add(a, b)).all(), ("add", m)
        elif op == B.OP_SUB:
            got = np.stack([out[d["r"][i]: d["r"][i] + m] for i in idx])
            r, s = oracle.sub(a, b)
            assert (got == r).all(), ("sub", m)
            assert (flags[d["flag"][idx]] == s).all(), ("sub sign", m)
        elif op == B.OP_MULFULL:
            got = np.stack([out[d["r"][i]: d["r"][i] + 2 * m] for i in idx])
            assert (got == oracle.mulfull(a, b, nthreads=nthreads)).all(), ("mulfull", m)
        elif op == B.OP_MUL:
            got = np.stack([out[d["r"][i]: d["r"][i] + m] for i in idx])
            assert (got == oracle.mul(a, b, nthreads=nthreads)).all(), ("mul", m)
        else:
            q = np.stack([out[d["r"][i]: d["r"][i] + m] for i in idx])
            r = np.stack([out[d["r2"][i]: d["r2"][i] + mb] for i in idx])
            qo, ro, so = oracle.div(a, b, nthreads=nthreads)
            assert (q == qo).all() and (r == ro).all(), ("div", m, mb)
            assert (flags[d["flag"][idx]] == so).all()


def _run(B, d, arena, out_limbs, nflags, tune=None, autotune=False):
    import torch

    din = B.to_device(arena)
    dout = torch.zeros(max(1, out_limbs), dtype=torch.int64, device="cuda")
    dfl = torch.zeros(max(1, nflags), dtype=torch.uint8, device="cuda")
    plan = B.Plan(d, len(arena), dout.numel(), dfl.numel())
    if tune:
        plan.set_tuning(*tune)
    if autotune:
        plan.autotune(din, dout, dfl, reps=1)
    plan.execute(din, dout, dfl)
    torch.cuda.synchronize()
    return plan, din, dout, dfl


def test_uneven_batch_small_sizes(bigint, oracle):
    B = bigint
    d, arena, out_limbs, nflags = B.workloads.uneven_batch(n=3000, seed=77, max_bits=8192)
    plan, din, dout, dfl = _run(B, d, arena, out_limbs, nflags)
    check_batch(B, oracle, d, arena, B.to_host(dout, np.uint64), dfl.cpu().numpy())
    st = plan.stats()
    assert st["addsub"] + st["mul"] + st["div"] == len(d)
    plan.close()


@pytest.mark.parametrize("tune", [(2, 2, 1), (8, 2, 2), (4, 1, 4)])
def test_tunings_agree(bigint, oracle, tune):
    B = bigint
    d, arena, out_limbs, nflags = B.workloads.uneven_batch(n=800, seed=78, max_bits=16384)
    plan, din, dout, dfl = _run(B, d, arena, out_limbs, nflags, tune=tune)
    check_batch(B, oracle, d, arena, B.to_host(dout, np.uint64), dfl.cpu().numpy())
    plan.close()


def test_autotune_then_replay_and_recapture(bigint, oracle):
    import torch

    B = bigint
    d, arena, out_limbs, nflags = B.workloads.uneven_batch(n=1500, seed=79, max_bits=4096)
    plan, din, dout, dfl = _run(B, d, arena, out_limbs, nflags, autotune=True)
    first = dout.clone()
    dout.zero_()
    plan.execute(din, dout, dfl)                  # graph replay
    torch.cuda.synchronize()
    assert bool((dout == first).all())
    dout2 = torch.zeros_like(dout)
    plan.execute(din, dout2, dfl)                 # new arena: recapture
    torch.cuda.synchronize()
    assert bool((dout2 == first).all())
    check_batch(B, oracle, d, arena, B.to_host(dout2, np.uint64), dfl.cpu().numpy())
    plan.close()


def test_large_instances(bigint, oracle):
    """The largest sizes the batch accepts, one op at a time, with unaligned offsets."""
    B = bigint
    rows = []
    arena = []
    off = 1                                       # odd limb offsets: the 8-byte path
    out = 0
    for op, m, mb in [(B.OP_ADD, 2048, 2048), (B.OP_SUB, 1500, 1500), (B.OP_MULFULL, 1024, 1024),
                      (B.OP_MUL, 2048, 2048), (B.OP_DIV, 2048, 1024), (B.OP_DIV, 1000, 3)]:
        a = B.workloads.uniform_limbs(500 + m + op, 1, m)[0]
        b = B.workloads.uniform_limbs(600 + m + op, 1, mb)[0]
        b[-1] |= np.uint64(1)
        rows.append((op, m, mb, off, off + m, out))
        arena += [a, b]
        off += m + mb
        out += 3 * m + mb
    d = np.zeros(len(rows), dtype=B.DESC_DTYPE)
    for i, (op, m, mb, ao, bo, ro) in enumerate(rows):
        d[i] = (op, m, mb, 0, ao, bo, ro, ro + (2 * m if op != B.OP_DIV else m), i)
    ar = np.concatenate([np.zeros(1, np.uint64)] + arena)
    plan, din, dout, dfl = _run(B, d, ar, out, len(d))
    check_batch(B, oracle, d, ar, B.to_host(dout, np.uint64), dfl.cpu().numpy())
    plan.close()


def test_division_classes_by_count(bigint, oracle):
    """Large-divisor classes run long division on warps when they hold many
    divisions and the shifted inverse on CTAs when they hold few: 400
    divisions of 400/200 limbs (above two per SM: warps) beside 6 of
    1200/600 limbs (CTAs) and 40 of 60/20 limbs (warps, always)."""
    B = bigint
    rows = []
    arena = []
    off = 0
    out = 0
    seed = 900
    for m, mb, count in [(400, 200, 400), (1200, 600, 6), (60, 20, 40)]:
        for _ in range(count):
            a = B.workloads.uniform_limbs(seed, 1, m)[0]
            b = B.workloads.uniform_limbs(seed + 1, 1, mb)[0]
            seed += 2
            b[-1] |= np.uint64(1)
            rows.append((m, mb, off, off + m, out))
            arena += [a, b]
            off += m + mb
            out += m + mb
    d = np.zeros(len(rows), dtype=B.DESC_DTYPE)
    for i, (m, mb, ao, bo, ro) in enumerate(rows):
        d[i] = (B.OP_DIV, m, mb, 0, ao, bo, ro, ro + m, i)
    ar = np.concatenate(arena)
    plan, din, dout, dfl = _run(B, d, ar, out, len(d))
    check_batch(B, oracle, d, ar, B.to_host(dout, np.uint64), dfl.cpu().numpy())
    plan.close()


def test_batch_matches_per_size_kernels(bigint):
    """The batch and the plain one-launch-per-size kernels give the same results."""
    import torch

    B = bigint
    d, arena, out_limbs, nflags = B.workloads.uneven_batch(n=2000, seed=80, max_bits=32768)
    plan, din, dout, dfl = _run(B, d, arena, out_limbs, nflags)
    out = B.to_host(dout, np.uint64)
    for (op, m, mb), idx in _groups(d).items():
        idx = np.array(idx)
        a = B.to_device(np.stack([arena[d["a"][i]: d["a"][i] + m] for i in idx]))
        b = B.to_device(np.stack([arena[d["b"][i]: d["b"][i] + mb] for i in idx]))
        if op == B.OP_ADD:
            ref = B.to_host(B.add(a, b), np.uint64)
            got = np.stack([out[d["r"][i]: d["r"][i] + m] for i in idx])
        elif op == B.OP_SUB:
            ref = B.to_host(B.sub(a, b)[0], np.uint64)
            got = np.stack([out[d["r"][i]: d["r"][i] + m] for i in idx])
        elif op == B.OP_MULFULL:
            ref = B.to_host(B.mulfull(a, b), np.uint64)
            got = np.stack([out[d["r"][i]: d["r"][i] + 2 * m] for i in idx])
        else:
            q, r, _ = B.div(a, b)
            ref = np.concatenate([B.to_host(q, np.uint64), B.to_host(r, np.uint64)], axis=1)
            got = np.stack([np.concatenate([out[d["r"][i]: d["r"][i] + m], out[d["r2"][i]: d["r2"][i] + mb]])
                            for i in idx])
        assert (got == ref).all(), (op, m)
    plan.close()
    torch.cuda.synchronize()


def test_full_size_batch_matches_per_size_kernels(bigint, oracle):
    """The benchmark's batch itself (100000 instances, 256..65536 bits, the
    mix and seed of the uneven-batch workload): every instance equals the
    plain per-size kernels' result; 3000 instances sampled across every op
    and size equal the oracle's (the per-size kernels and the batch share
    their multiply and division cores, so this catches a defect common to
    both); and a sample of the divisions satisfies u = q v + r with r < v in
    Python integers."""
    import os

    import torch

    B = bigint
    d, arena, out_limbs, nflags = B.workloads.uneven_batch()
    plan, din, dout, dfl = _run(B, d, arena, out_limbs, nflags)
    out = B.to_host(dout, np.uint64)
    flags = dfl.cpu().numpy()
    sample = np.sort(np.random.default_rng(7).choice(len(d), size=3000, replace=False))
    check_batch(B, oracle, d[sample], arena, out, flags, nthreads=os.cpu_count() or 1)

    def rows(src, off, idx, width):
        return src[d[off][idx].astype(np.int64)[:, None] + np.arange(width)]

    checked_div = 0
    for (op, m, mb), idx in _groups(d).items():
        idx = np.array(idx)
        a, b = rows(arena, "a", idx, m), rows(arena, "b", idx, mb)
        da, db = B.to_device(a), B.to_device(b)
        if op == B.OP_ADD:
            assert (rows(out, "r", idx, m) == B.to_host(B.add(da, db), np.uint64)).all(), ("add", m)
        elif op == B.OP_SUB:
            assert (rows(out, "r", idx, m) == B.to_host(B.sub(da, db)[0], np.uint64)).all(), ("sub", m)
        elif op == B.OP_MULFULL:
            assert (rows(out, "r", idx, 2 * m) == B.to_host(B.mulfull(da, db), np.uint64)).all(), ("mulfull", m)
        else:
            q, r, _ = B.div(da, db)
            gq, gr = rows(out, "r", idx, m), rows(out, "r2", idx, mb)
            assert (gq == B.to_host(q, np.uint64)).all() and (gr == B.to_host(r, np.uint64)).all(), ("div", m)
            if checked_div < 200:
                k = 0
                to_int = lambda limbs: sum(int(x) << (64 * i) for i, x in enumerate(limbs))
                U, V, Q, R = to_int(a[k]), to_int(b[k]), to_int(gq[k]), to_int(gr[k])
                assert U == Q * V + R and R < V, ("div identity", m, mb)
                checked_div += 1
    assert checked_div > 50
    plan.close()
    torch.cuda.synchronize()


def test_invalid_descriptors_rejected(bigint):
    B = bigint
    d = np.zeros(1, dtype=B.DESC_DTYPE)
    for bad in [dict(op=0, m=0, mb=0), dict(op=9, m=4, mb=4), dict(op=4, m=4, mb=5), dict(op=0, m=5000, mb=5000)]:
        d[0]["op"], d[0]["m"], d[0]["mb"] = bad["op"], bad["m"], bad["mb"]
        with pytest.raises(B.BigIntError):
            B.Plan(d, 1 << 20, 1 << 20, 16)
    empty = B.Plan(np.zeros(0, dtype=B.DESC_DTYPE), 0, 0)
    assert empty.stats()["addsub"] == 0
    empty.close()


def _small_mul_batch(B, n=600, seed=91):
    """Full products of 1..32 limbs (every warp class, odd sizes), with some
    truncated and larger full products and additions between them."""
    rng = np.random.default_rng(seed)
    d = np.zeros(n, dtype=B.DESC_DTYPE)
    pos = 0
    out = 0
    for i in range(n):
        kind = i % 6
        m = int(rng.integers(1, 33)) if kind < 4 else int(rng.integers(33, 80))
        op = B.OP_MULFULL if kind in (0, 1, 2, 4) else (B.OP_MUL if kind == 3 else B.OP_ADD)
        d[i]["op"], d[i]["m"], d[i]["mb"] = op, m, m
        d[i]["a"], d[i]["b"] = pos, pos + m
        pos += 2 * m
        d[i]["r"] = out
        out += 2 * m if op == B.OP_MULFULL else m
    arena = rng.integers(0, 2**64, size=pos, dtype=np.uint64)
    arena[: 2 * 32] = np.uint64(0xFFFFFFFFFFFFFFFF)      # the first operands all ones
    return d, arena, out, 1


@pytest.mark.parametrize("bits", [32, 64])
def test_small_full_products_at_either_word_width(bigint, oracle, bits):
    """The plan's full products of at most 32 limbs run on 32-bit words (the
    warp kernel) or on 64-bit limbs (the CTA kernel): the same products."""
    import torch

    B = bigint
    d, arena, out_limbs, nflags = _small_mul_batch(B)
    din = B.to_device(arena)
    dout = torch.zeros(out_limbs, dtype=torch.int64, device="cuda")
    dfl = torch.zeros(1, dtype=torch.uint8, device="cuda")
    plan = B.Plan(d, len(arena), out_limbs, 1)
    plan.set_mul_word_bits(bits)
    assert plan.tuning()["mul_small_word_bits"] == bits
    plan.execute(din, dout, dfl)
    torch.cuda.synchronize()
    check_batch(B, oracle, d, arena, B.to_host(dout, np.uint64), dfl.cpu().numpy())
    with pytest.raises(B.BigIntError):
        plan.set_mul_word_bits(48)
    plan.close()


def test_autotune_picks_a_word_width(bigint, oracle):
    import torch

    B = bigint
    d, arena, out_limbs, nflags = _small_mul_batch(B, n=900, seed=92)
    din = B.to_device(arena)
    dout = torch.zeros(out_limbs, dtype=torch.int64, device="cuda")
    dfl = torch.zeros(1, dtype=torch.uint8, device="cuda")
    plan = B.Plan(d, len(arena), out_limbs, 1)
    t = plan.autotune(din, dout, dfl, reps=1)
    assert t["mul_small_word_bits"] in (32, 64) and t == plan.tuning()
    dout.zero_()
    plan.execute(din, dout, dfl)
    torch.cuda.synchronize()
    check_batch(B, oracle, d, arena, B.to_host(dout, np.uint64), dfl.cpu().numpy())
    plan.close()


def test_large_divisions_in_a_batch(bigint, oracle):
    """Divisions beyond the one-limb-per-step kernels' reach inside a mixed
    batch: divisors of 1025..4096 limbs (block long division on two and four
    warps) with dividends up to 8192 limbs, and a few 500-1000-limb divisors
    of dividends longer than the shifted inverse takes (they stay on long
    division), beside additions and products."""
    B = bigint
    rng = np.random.default_rng(77)
    shapes = [(2100, 1025), (4000, 2048), (4100, 2049), (8192, 4096), (3000, 1500), (3000, 600), (2500, 900)]
    ops = [(B.OP_DIV, m, mb) for m, mb in shapes] + [(B.OP_ADD, 300, 300), (B.OP_MULFULL, 200, 200),
                                                     (B.OP_SUB, 64, 64), (B.OP_DIV, 40, 20)]
    d = np.zeros(len(ops), dtype=B.DESC_DTYPE)
    pos = out = 0
    for i, (op, m, mb) in enumerate(ops):
        d[i]["op"], d[i]["m"], d[i]["mb"] = op, m, mb
        d[i]["a"], d[i]["b"] = pos, pos + m
        pos += m + mb
        d[i]["r"] = out
        out += 2 * m if op == B.OP_MULFULL else m
        if op == B.OP_DIV:
            d[i]["r2"] = out
            out += mb
        d[i]["flag"] = i
    arena = rng.integers(0, 2**64, size=pos, dtype=np.uint64)
    for i, (op, m, mb) in enumerate(ops):
        if op == B.OP_DIV:
            arena[d[i]["b"] + mb - 1] |= np.uint64(1 << 63)
    arena[d[1]["a"]: d[1]["a"] + 4000] = np.uint64(0xFFFFFFFFFFFFFFFF)   # an all-ones dividend
    plan, din, dout, dfl = _run(B, d, arena, out, len(ops))
    import os
    check_batch(B, oracle, d, arena, B.to_host(dout, np.uint64), dfl.cpu().numpy(), nthreads=os.cpu_count() or 1)
    plan.close()


def test_division_lane_classes_in_a_batch(bigint):
    """Divisions of 2m by m limbs for divisors on either side of the batch's
    lane-width classes (16-lane groups of 24 limbs up to 384, warps of 16
    limbs up to 512, of 24 up to 768 and of 32 up to 1024), enough of each
    class that none runs as the shifted inverse; checked as Python
    integers (u = q v + r, r < v)."""
    B = bigint
    rng = np.random.default_rng(91)
    shapes = [(mv, 160) for mv in (257, 300, 384, 385, 450, 512)] + [(mv, 310) for mv in (513, 600, 768, 769, 900, 1024)]
    ops = [mv for mv, k in shapes for _ in range(k)]
    d = np.zeros(len(ops), dtype=B.DESC_DTYPE)
    pos = out = 0
    for i, mv in enumerate(ops):
        m = 2 * mv
        d[i]["op"], d[i]["m"], d[i]["mb"] = B.OP_DIV, m, mv
        d[i]["a"], d[i]["b"] = pos, pos + m
        pos += m + mv
        d[i]["r"], d[i]["r2"] = out, out + m
        out += m + mv
        d[i]["flag"] = i
    arena = rng.integers(0, 2**64, size=pos, dtype=np.uint64)
    for i, mv in enumerate(ops):
        b = int(d[i]["b"])
        arena[b + mv - 1] |= np.uint64(1)
        if i % 97 == 0:                                   # all-ones operands
            arena[int(d[i]["a"]): b + mv] = np.uint64(0xFFFFFFFFFFFFFFFF)
    plan, din, dout, dfl = _run(B, d, arena, out, len(ops))
    res = B.to_host(dout, np.uint64)
    assert (dfl.cpu().numpy()[: len(ops)] == 0).all()
    for i, mv in enumerate(ops):
        a, b, r, r2 = int(d[i]["a"]), int(d[i]["b"]), int(d[i]["r"]), int(d[i]["r2"])
        U = int.from_bytes(arena[a: a + 2 * mv].tobytes(), "little")
        V = int.from_bytes(arena[b: b + mv].tobytes(), "little")
        Q = int.from_bytes(res[r: r + 2 * mv].tobytes(), "little")
        R = int.from_bytes(res[r2: r2 + mv].tobytes(), "little")
        assert Q * V + R == U and R < V, (mv, i)
    plan.close()


def test_batch_size_limits_rejected(bigint):
    """Sizes past the batch's limits are refused when the plan is built."""
    B = bigint
    for op, m, mb in [(B.OP_ADD, 2049, 2049), (B.OP_MULFULL, 2049, 2049), (B.OP_DIV, 8193, 100),
                      (B.OP_DIV, 8192, 4097)]:
        d = np.zeros(1, dtype=B.DESC_DTYPE)
        d[0]["op"], d[0]["m"], d[0]["mb"] = op, m, mb
        d[0]["b"] = m
        with pytest.raises(B.BigIntError) as ei:
            B.Plan(d, 1 << 20, 1 << 20, 16)
        assert ei.value.status == 6             # BI_EUNSUPPORTED



def _mixed_width_batch(B, n=1200, seed=55):
    """A batch mixing 64-bit-limb instances (width 0) and 32-bit-word ones
    (width 32) of every op: odd and even word counts, odd and even word
    offsets, all-ones operands, divisors of every class up to 1100 words."""
    rng = np.random.default_rng(seed)
    ops = [B.OP_ADD, B.OP_SUB, B.OP_MUL, B.OP_MULFULL, B.OP_DIV]
    d = np.zeros(n, dtype=B.DESC_DTYPE)
    pos64 = out64 = 0
    rows = []
    for i in range(n):
        op = ops[i % 5]
        w32 = (i // 5) % 3 != 0
        m = int(rng.integers(1, 2200 if op == B.OP_DIV else 300))
        if op == B.OP_MULFULL and i % 7 == 0:
            m = int(rng.integers(1, 65))                 # the warp-multiply classes
        mb = int(rng.integers(1, m + 1)) if op == B.OP_DIV else m
        rows.append((op, m, mb, w32))
    # 64-bit instances first (limb offsets), then the word instances (word offsets, some odd)
    for i, (op, m, mb, w32) in enumerate(rows):
        if w32:
            continue
        d[i]["op"], d[i]["m"], d[i]["mb"], d[i]["width"] = op, m, mb, 0
        d[i]["a"], d[i]["b"] = pos64, pos64 + m
        pos64 += m + mb
        d[i]["r"] = out64
        out64 += 2 * m if op == B.OP_MULFULL else m
        if op == B.OP_DIV:
            d[i]["r2"] = out64
            out64 += mb
    pw, ow = 2 * pos64 + 1, 2 * out64 + 3               # word cursors, starting odd
    for i, (op, m, mb, w32) in enumerate(rows):
        if not w32:
            continue
        d[i]["op"], d[i]["m"], d[i]["mb"], d[i]["width"] = op, m, mb, 32
        d[i]["a"], d[i]["b"] = pw, pw + m
        pw += m + mb + (i & 1)
        d[i]["r"] = ow
        ow += 2 * m if op == B.OP_MULFULL else m
        if op == B.OP_DIV:
            d[i]["r2"] = ow
            ow += mb
        ow += i & 1
    d["flag"] = np.arange(n)
    in_limbs, out_limbs = (pw + 1) // 2 + 1, (ow + 1) // 2 + 1
    arena = rng.integers(0, 2**64, size=in_limbs, dtype=np.uint64)
    a32 = arena.view(np.uint32)
    for i, (op, m, mb, w32) in enumerate(rows):
        view, off = (a32, int(d[i]["b"])) if w32 else (arena, int(d[i]["b"]))
        if op == B.OP_DIV:
            view[off + mb - 1] |= view.dtype.type(1)    # nonzero top divisor element
        if i % 11 == 0:                                  # all-ones operands
            oa = int(d[i]["a"])
            view[oa: oa + m] = np.iinfo(view.dtype).max
    return d, arena, out_limbs, n


def test_mixed_width_batch_matches_oracle(bigint, oracle):
    """32-bit-word instances (the reference's U32bits layout) in the same
    batch as 64-bit-limb ones, each checked against the oracle on its own
    element type."""
    import os

    import torch

    B = bigint
    d, arena, out_limbs, nflags = _mixed_width_batch(B)
    plan, din, dout, dfl = _run(B, d, arena, out_limbs, nflags)
    out = B.to_host(dout, np.uint64)
    flags = dfl.cpu().numpy()
    th = os.cpu_count() or 1
    for w, a_view, o_view in ((0, arena, out), (32, arena.view(np.uint32), out.view(np.uint32))):
        sel = np.nonzero(d["width"] == w)[0]
        assert sel.size > 100
        check_batch(B, oracle, d[sel], a_view, o_view, flags, nthreads=th)
    plan.close()
