"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``liboracle.so`` (the C restatement in ``bigint_oracle.c``) and, where
it was built, ``_ref/libref_div.so`` (the reference's own
``prototypes/div.c``).  Only the tests, the smoke check and the benchmark's
CPU-baseline and reference legs import this module; the library never does.

All arrays are numpy, C-contiguous, shape ``[n, m]`` of ``uint32`` or
``uint64`` little-endian limbs.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "liboracle.so")
_REF_DIV = os.path.join(HERE, "_ref", "libref_div.so")

_lib = None
_ref = None


def reference_checkout():
    """The reference checkout whose prototypes/div.c is compiled beside the
    oracle: $BIGINT_REF, else a `reference` directory beside the
    repository; None when neither exists."""
    for cand in (os.environ.get("BIGINT_REF"), os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")):
        if cand and os.path.isdir(cand):
            return cand
    return None


def build(quiet: bool = True) -> None:
    """Compile the oracle (and the reference's div.c where present)."""
    ref = reference_checkout()
    out = subprocess.run(["make", "-C", HERE, "all"] + ([f"REF={ref}"] if ref else []), capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(
            os.path.join(HERE, "bigint_oracle.c")
        ):
            build()
        L = ctypes.CDLL(_LIB)
        P, U32, U64, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        for w in ("u32", "u64"):
            for op in ("add", "mul", "mulfull"):
                f = getattr(L, f"orc_{op}_{w}")
                f.argtypes = [P, P, P, U32, U64, I]
                f.restype = I
            f = getattr(L, f"orc_sub_{w}")
            f.argtypes = [P, P, P, P, U32, U64, I]
            f.restype = I
            f = getattr(L, f"orc_div_{w}")
            f.argtypes = [P, P, P, P, P, U32, U32, U64, I]
            f.restype = I
        L.orc_div_ref_u32.argtypes = [P, P, P, P, P, U32, U32, U64, I]
        L.orc_div_ref_u32.restype = I
        L.orc_div_ref_word_products_u32.argtypes = [P, P, U32]
        L.orc_div_ref_word_products_u32.restype = U64
        L.orc_little_endian.restype = I
        if L.orc_little_endian() != 1:
            raise RuntimeError("oracle requires a little-endian host")
        _lib = L
    return _lib


def ref_div_lib():
    """The reference's prototypes/div.c as a shared library, or None."""
    global _ref
    if _ref is None and os.path.exists(_REF_DIV):
        R = ctypes.CDLL(_REF_DIV)
        R.div_shinv.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int]
        R.div_shinv.restype = None
        _ref = R
    return _ref


def _wname(a: np.ndarray) -> str:
    if a.dtype == np.uint32:
        return "u32"
    if a.dtype == np.uint64:
        return "u64"
    raise TypeError(f"limbs must be uint32 or uint64, got {a.dtype}")


def _c(a):
    return np.ascontiguousarray(a)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def add(a, b, nthreads: int = 1):
    a, b = _c(a), _c(b)
    n, m = a.shape
    r = np.empty_like(a)
    getattr(lib(), f"orc_add_{_wname(a)}")(_p(a), _p(b), _p(r), m, n, nthreads)
    return r


def sub(a, b, nthreads: int = 1):
    a, b = _c(a), _c(b)
    n, m = a.shape
    r = np.empty_like(a)
    s = np.empty(n, dtype=np.uint8)
    getattr(lib(), f"orc_sub_{_wname(a)}")(_p(a), _p(b), _p(r), _p(s), m, n, nthreads)
    return r, s


def mul(a, b, nthreads: int = 1):
    a, b = _c(a), _c(b)
    n, m = a.shape
    r = np.empty_like(a)
    getattr(lib(), f"orc_mul_{_wname(a)}")(_p(a), _p(b), _p(r), m, n, nthreads)
    return r


def mulfull(a, b, nthreads: int = 1):
    a, b = _c(a), _c(b)
    n, m = a.shape
    r = np.empty((n, 2 * m), dtype=a.dtype)
    getattr(lib(), f"orc_mulfull_{_wname(a)}")(_p(a), _p(b), _p(r), m, n, nthreads)
    return r


def div(u, v, nthreads: int = 1):
    """(q, r, status): q [n][mu], r [n][mv]; status[i] = 1 where v_i == 0."""
    u, v = _c(u), _c(v)
    n, mu = u.shape
    mv = v.shape[1]
    q = np.empty_like(u)
    r = np.empty((n, mv), dtype=u.dtype)
    st = np.zeros(n, dtype=np.uint8)
    getattr(lib(), f"orc_div_{_wname(u)}")(_p(u), _p(v), _p(q), _p(r), _p(st), mu, mv, n, nthreads)
    return q, r, st


def div_ref(u, v, nthreads: int = 1):
    """The reference's division algorithm exactly as written (u32 digits,
    single delta step, so occasionally one short -- see bigint_oracle.c)."""
    u = _c(u).astype(np.uint32, copy=False)
    v = _c(v).astype(np.uint32, copy=False)
    n, mu = u.shape
    mv = v.shape[1]
    q = np.empty_like(u)
    r = np.empty((n, mv), dtype=np.uint32)
    st = np.zeros(n, dtype=np.uint8)
    lib().orc_div_ref_u32(_p(u), _p(v), _p(q), _p(r), _p(st), mu, mv, n, nthreads)
    return q, r, st


def div_ref_word_products(u, v) -> int:
    """32x32-bit word products of the multiplications the reference's
    division (div.c's div_shinv, as div_ref runs it) performs on one
    instance: u a 1-D array of u32 digits (or u64 limbs, read as u32 pairs),
    v the divisor, zero-extended to u's digits as div.c requires; counted on
    significant digits as GMP's mpz_mul multiplies them."""
    u = np.ascontiguousarray(np.asarray(u).reshape(-1)).view(np.uint32)
    v = np.ascontiguousarray(np.asarray(v).reshape(-1)).view(np.uint32)
    m = u.shape[0]
    vp = np.zeros(m, dtype=np.uint32)
    vp[: v.shape[0]] = v
    return int(lib().orc_div_ref_word_products_u32(_p(u), _p(vp), m))


def ref_div_u32(u, v):
    """Run the reference's own div_shinv (u32 digits, equal sizes) per row."""
    R = ref_div_lib()
    if R is None:
        raise RuntimeError("reference div.c was not built (needs the reference checkout and libgmp)")
    u = _c(u).astype(np.uint32, copy=False)
    v = _c(v).astype(np.uint32, copy=False)
    n, m = u.shape
    q = np.zeros_like(u)
    r = np.zeros_like(u)
    for i in range(n):
        ui, vi = np.ascontiguousarray(u[i]), np.ascontiguousarray(v[i])
        qi, ri = np.zeros(m, np.uint32), np.zeros(m, np.uint32)
        R.div_shinv(_p(ui), _p(vi), _p(qi), _p(ri), m)
        q[i], r[i] = qi, ri
    return q, r


# ---- conversions used by tests ------------------------------------------

def to_int(row) -> int:
    """Little-endian limb row -> Python int."""
    row = np.asarray(row)
    bits = row.dtype.itemsize * 8
    return int.from_bytes(row.astype(row.dtype.newbyteorder("<")).tobytes(), "little") if bits else 0


def from_int(x: int, m: int, dtype=np.uint64) -> np.ndarray:
    """Python int (reduced mod B^m) -> little-endian limb row of length m."""
    nbytes = m * np.dtype(dtype).itemsize
    x &= (1 << (8 * nbytes)) - 1
    return np.frombuffer(x.to_bytes(nbytes, "little"), dtype=np.dtype(dtype).newbyteorder("<")).astype(dtype)


# ---- the division prototype's helper primitives (pure Python, small cases) --
# Restated from prototypes/div.c on digit arrays of either width; rows of a
# [n][m] batch are processed one by one.

def cmp_rows(a, b) -> np.ndarray:
    """-1, 0, 1 per row as a <, ==, > b: lt and eq (div.c:49-62)."""
    out = np.zeros(a.shape[0], np.int8)
    for i in range(a.shape[0]):
        res = 0
        for j in range(a.shape[1]):          # lt's loop: the last difference decides
            if a[i, j] != b[i, j]:
                res = -1 if a[i, j] < b[i, j] else 1
        out[i] = res
    return out


def findk_rows(a):
    """(k, zero) per row: findk (div.c:92-96) and ez (div.c:64-69)."""
    k = np.zeros(a.shape[0], np.int64)
    z = np.zeros(a.shape[0], np.uint8)
    for i in range(a.shape[0]):
        kk = 0
        for j in range(a.shape[1]):
            kk = j if a[i, j] != 0 else kk
        k[i] = kk
        z[i] = 1 if not a[i].any() else 0
    return k, z


def shift_rows(a, n: int):
    """shift (div.c:104-117): n >= 0 moves digits up, n < 0 down."""
    m = a.shape[1]
    r = np.zeros_like(a)
    for j in range(m):
        src = j - n
        if 0 <= src < m:
            r[:, j] = a[:, src]
    return r


def muld_rows(a, d):
    """multd (div.c:197-217): a * d mod B^m with one digit d per row."""
    m = a.shape[1]
    out = np.zeros_like(a)
    for i in range(a.shape[0]):
        out[i] = from_int(to_int(a[i]) * int(d[i]), m, a.dtype)
    return out


def quod_rows(a, d):
    """quod (div.c:165-181): long division by one digit d per row; also the
    remainder.  d = 0 gives 0 and 0."""
    m = a.shape[1]
    bits = a.dtype.itemsize * 8
    q = np.zeros_like(a)
    rem = np.zeros(a.shape[0], a.dtype)
    for i in range(a.shape[0]):
        dd = int(d[i])
        if dd == 0:
            continue
        r = 0
        for j in range(m - 1, -1, -1):       # top digit first, as div.c
            r = (r << bits) + int(a[i, j])
            q[i, j] = r // dd
            r -= (r // dd) * dd
        rem[i] = r
    return q, rem
