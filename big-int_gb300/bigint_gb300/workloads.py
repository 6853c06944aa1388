"""Seeded synthetic inputs with the shapes of the benchmarked workloads.

The reference benchmarks on unseeded ``rand()`` digits (cuda/helpers.h:96-111);
here every input comes from a splitmix64 stream so runs are reproducible on
any machine.  Seeds are 1000 + the workload index:

  * mul2048_u32  -- 4096 pairs of 64-limb u32 integers (2048 bits), 10 % of
                    pairs all-0xFFFFFFFF; full 128-limb product.
  * addsub_u64   -- u64 limbs, sizes 2^10..2^18 bits, n = 2^27 / m instances;
                    80 % uniform, 20 % carry-chain instances (add: a low run
                    of all-ones limbs of length L in [m/2, m], b's low limb
                    odd; sub: a low run of zero limbs, b = 1).
  * mul_u64      -- u64 limbs, m in {64, 256, 1024, 2048}, n in
                    {2^16, 2^14, 2^12, 2^11}, uniform; full 2m-limb product.
  * uneven_batch -- 100k instances, sizes log-uniform over 256..65536 bits
                    (u64 limbs), ops 20 % add, 20 % sub, 40 % full multiply,
                    20 % division (dividend 2m limbs, divisor m limbs with a
                    nonzero top limb); seed 1003.
"""
from __future__ import annotations

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """``count`` outputs of the splitmix64 stream ``seed``, starting at ``offset``."""
    with np.errstate(over="ignore"):
        idx = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform_limbs(seed: int, n: int, m: int, dtype=np.uint64, offset: int = 0) -> np.ndarray:
    if dtype == np.uint64:
        return splitmix64(seed, n * m, offset).reshape(n, m)
    if dtype == np.uint32:
        w = splitmix64(seed, (n * m + 1) // 2, offset).view(np.uint32)[: n * m]
        return w.reshape(n, m).copy()
    raise TypeError(dtype)


def pick(seed: int, n: int, frac: float) -> np.ndarray:
    """Boolean mask selecting about ``frac`` of ``n`` instances."""
    u = splitmix64(seed ^ 0x5EED, n) >> np.uint64(11)
    return (u.astype(np.float64) * (1.0 / (1 << 53))) < frac


# ---------------------------------------------------------------------------

def mul2048_u32(seed: int = 1000, n: int = 4096, m: int = 64):
    a = uniform_limbs(seed, n, m, np.uint32)
    b = uniform_limbs(seed, n, m, np.uint32, offset=(n * m + 1) // 2)
    ones = pick(seed, n, 0.10)
    a[ones] = 0xFFFFFFFF
    b[ones] = 0xFFFFFFFF
    return a, b


ADDSUB_BITS = [1 << k for k in range(10, 19)]   # 2^10 .. 2^18 bits


def _chains(bits: int, seed: int, n: int, m: int):
    """Indices of the carry-chain instances and their run lengths in [m/2, m]."""
    chain = np.nonzero(pick(seed + bits, n, 0.20))[0]
    lens = m // 2 + (splitmix64(seed + 7 * bits, chain.size) % np.uint64(m - m // 2 + 1)).astype(np.int64)
    return chain, lens


def addsub_u64(bits: int, seed: int = 1001, total_limbs: int = 1 << 27, op: str = "add"):
    """Inputs for one size of the add/sub sweep (u64 limbs, n*m = total_limbs)."""
    m = bits // 64
    n = total_limbs // m
    a = uniform_limbs(seed, n, m)
    b = uniform_limbs(seed, n, m, offset=n * m)
    chain, lens = _chains(bits, seed, n, m)
    if chain.size:
        cols = np.arange(m)[None, :]
        run = cols < lens[:, None]
        if op == "add":
            rows = a[chain]
            rows[run] = np.uint64(0xFFFFFFFFFFFFFFFF)
            a[chain] = rows
            b[chain, 0] |= np.uint64(1)
        else:
            rows = a[chain]
            rows[run] = np.uint64(0)
            a[chain] = rows
            b[chain] = 0
            b[chain, 0] = 1
    return a, b


MUL_U64 = [(64, 1 << 16), (256, 1 << 14), (1024, 1 << 12), (2048, 1 << 11)]


def mul_u64(m: int, n: int, seed: int = 1002):
    a = uniform_limbs(seed, n, m)
    b = uniform_limbs(seed, n, m, offset=n * m)
    return a, b


# ---------------------------------------------------------------------------
# Device-side generation (same values as above, built on the GPU with the
# library's splitmix64 fill kernel; tensors are int64 holding u64 limb bits)
# ---------------------------------------------------------------------------

def device_uniform_u64(seed: int, n: int, m: int, offset: int = 0, device="cuda"):
    import torch

    from . import fill_splitmix64

    t = torch.empty((n, m), dtype=torch.int64, device=device)
    fill_splitmix64(t, seed, offset)
    return t


def addsub_u64_device(bits: int, seed: int = 1001, total_limbs: int = 1 << 27, op: str = "add",
                      device="cuda"):
    import torch

    m = bits // 64
    n = total_limbs // m
    a = device_uniform_u64(seed, n, m, device=device)
    b = device_uniform_u64(seed, n, m, offset=n * m, device=device)
    chain, lens = _chains(bits, seed, n, m)
    if chain.size:
        ci = torch.from_numpy(chain).to(device)
        run = torch.arange(m, device=device)[None, :] < torch.from_numpy(lens).to(device)[:, None]
        rows = a[ci]
        if op == "add":
            rows[run] = -1
            a[ci] = rows
            b[ci, 0] |= 1
        else:
            rows[run] = 0
            a[ci] = rows
            b[ci] = 0
            b[ci, 0] = 1
    return a, b


def mul_u64_device(m: int, n: int, seed: int = 1002, device="cuda"):
    return (device_uniform_u64(seed, n, m, device=device),
            device_uniform_u64(seed, n, m, offset=n * m, device=device))


def uneven_batch(n: int = 100_000, seed: int = 1003, min_bits: int = 256, max_bits: int = 65536):
    """Descriptors and input arena of the uneven-size batch.

    Returns (descs, arena_in, out_limbs, flag_bytes): descs is a DESC_DTYPE
    array, arena_in a uint64 array holding every operand back to back in
    descriptor order; outputs go to an arena of out_limbs limbs (per
    instance: m for add/sub, 2m for the full product, 2m quotient + m
    remainder for division) and a flag arena of flag_bytes bytes.
    """
    from . import DESC_DTYPE, OP_ADD, OP_DIV, OP_MULFULL, OP_SUB

    u = (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    lo, hi = np.log2(min_bits), np.log2(max_bits)
    bits = np.exp2(lo + (hi - lo) * u)
    m = np.maximum(1, np.ceil(bits / 64.0)).astype(np.int64)
    sel = (splitmix64(seed + 1, n) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    op = np.where(sel < 0.2, OP_ADD, np.where(sel < 0.4, OP_SUB, np.where(sel < 0.8, OP_MULFULL, OP_DIV)))
    ma = np.where(op == OP_DIV, 2 * m, m)           # first operand limbs
    mb = m                                          # second operand limbs
    a_off = np.zeros(n, np.int64)
    a_off[1:] = np.cumsum(ma + mb)[:-1]
    b_off = a_off + ma
    rl = np.where(op == OP_ADD, m, np.where(op == OP_SUB, m, 2 * m))   # q has the dividend's 2m limbs
    r2l = np.where(op == OP_DIV, m, 0)
    r_off = np.zeros(n, np.int64)
    r_off[1:] = np.cumsum(rl + r2l)[:-1]
    total_in = int((ma + mb).sum())
    arena = splitmix64(seed + 2, total_in)
    div_idx = np.nonzero(op == OP_DIV)[0]
    top = b_off[div_idx] + mb[div_idx] - 1          # divisor top limb nonzero
    arena[top] |= np.uint64(1)
    d = np.zeros(n, dtype=DESC_DTYPE)
    d["op"] = op
    d["m"] = ma
    d["mb"] = mb
    d["a"] = a_off
    d["b"] = b_off
    d["r"] = r_off
    d["r2"] = r_off + rl
    d["flag"] = np.arange(n)
    return d, arena, int((rl + r2l).sum()), n


# ---------------------------------------------------------------------------
# serving stream: Poisson arrivals of add/sub/mul/div requests
# ---------------------------------------------------------------------------

SERVE_RATES = [10_000, 30_000, 100_000, 300_000, 1_000_000]   # offered requests/s


def _unit(seed: int, n: int) -> np.ndarray:
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) / float(1 << 53)


def serve_stream(n: int, rate: float, seed: int = 1004, pool_limbs: int = 1 << 22, min_bits: int = 512,
                 max_bits: int = 32768, mix=(0.15, 0.15, 0.40, 0.30)):
    """Requests and arrival times of the serving benchmark.

    Operand sizes are log-uniform in [min_bits, max_bits] (m = ceil(bits/64)
    64-bit limbs); the operation is add, sub, full multiply or division with
    the probabilities `mix`; a division divides the drawn size by a divisor
    of half as many limbs.  Operands are windows at even limb offsets of one
    shared pool of `pool_limbs` random limbs (splitmix64 stream seed + 5,
    resident on the device).  Arrivals form a Poisson process of `rate`
    requests/s.  Returns (descs, arrival_ns, pool_seed).
    """
    from . import DESC_DTYPE, OP_ADD, OP_DIV, OP_MULFULL, OP_SUB

    lo, hi = np.log2(min_bits), np.log2(max_bits)
    bits = np.exp2(lo + (hi - lo) * _unit(seed, n))
    m = np.maximum(1, np.ceil(bits / 64.0)).astype(np.int64)
    sel = _unit(seed + 1, n)
    c = np.cumsum(mix) / np.sum(mix)
    op = np.where(sel < c[0], OP_ADD, np.where(sel < c[1], OP_SUB, np.where(sel < c[2], OP_MULFULL, OP_DIV)))
    mb = np.where(op == OP_DIV, np.maximum(1, m // 2), m)
    a = 2 * np.floor(_unit(seed + 2, n) * ((pool_limbs - m) // 2 + 1)).astype(np.int64)
    b = 2 * np.floor(_unit(seed + 3, n) * ((pool_limbs - mb) // 2 + 1)).astype(np.int64)
    gaps = -np.log1p(-_unit(seed + 4, n)) / float(rate)
    arrival_ns = np.round(np.cumsum(gaps) * 1e9).astype(np.uint64)
    d = np.zeros(n, dtype=DESC_DTYPE)
    d["op"] = op
    d["m"] = m
    d["mb"] = mb
    d["a"] = a
    d["b"] = b
    return d, arrival_ns, seed + 5


def serve_pool_device(pool_limbs: int, pool_seed: int, device="cuda"):
    import torch

    from . import fill_splitmix64

    t = torch.empty(pool_limbs, dtype=torch.int64, device=device)
    fill_splitmix64(t, pool_seed, 0)
    return t
