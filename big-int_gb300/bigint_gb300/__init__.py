"""Python front end of the GB300 batched big-integer library.

A thin ctypes layer over ``libbigint_gb300.so`` (the C ABI declared in
``include/bigint_gb300.h``).  It exists for tests, benchmarks and Python
callers; C, C++ and other FFI users bind the shared library directly.

Device functions take CUDA tensors of shape ``[n, m]`` whose element size is 4
(u32 limbs) or 8 (u64 limbs) -- any integer dtype of that size, e.g.
``torch.int64`` holding the bits of u64 limbs -- and run on the current torch
stream unless ``stream`` is given.  Host functions take numpy ``uint32`` /
``uint64`` arrays and mirror the reference's synchronous host wrappers.

There is no CPU fallback: if the shared library is missing or fails to load,
every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _build
from . import workloads  # noqa: F401  (seeded synthetic inputs)

LIB_PATH = _build.LIB_PATH

_lib = None

STATUS = {
    0: "BI_OK",
    1: "BI_EINVAL",
    2: "BI_EDIV0",
    3: "BI_ENOMEM",
    4: "BI_ETIMEDOUT",
    5: "BI_ECUDA",
    6: "BI_EUNSUPPORTED",
}


class BigIntError(RuntimeError):
    def __init__(self, status: int, detail: str):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {detail}")


def build(force: bool = False, verbose: bool = False) -> str:
    return _build.build(force=force, verbose=verbose)


def lib() -> ctypes.CDLL:
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with bigint_gb300.build() "
            "(there is no CPU fallback)"
        )
    L = ctypes.CDLL(LIB_PATH)
    _declare(L)
    _lib = L
    return L


_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_I = ctypes.c_int

# name -> argtypes; every function returns int (bi_status) unless listed in _RESTYPE
SIGNATURES: dict[str, list] = {
    "bi_add_u64": [_P, _P, _P, _U32, _U64, _P],
    "bi_add_u32": [_P, _P, _P, _U32, _U64, _P],
    "bi_sub_u64": [_P, _P, _P, _P, _U32, _U64, _P],
    "bi_sub_u32": [_P, _P, _P, _P, _U32, _U64, _P],
    "bi_host_add_u64": [_P, _P, _P, _U32, _U64],
    "bi_host_add_u32": [_P, _P, _P, _U32, _U64],
    "bi_host_sub_u64": [_P, _P, _P, _P, _U32, _U64],
    "bi_host_sub_u32": [_P, _P, _P, _P, _U32, _U64],
    "bi_status_string": [_I],
    "bi_last_error": [],
    "bi_version": [],
    "bi_max_limbs_addsub_u64": [],
    "bi_max_limbs_addsub_u32": [],
    "bi_fill_splitmix64": [_P, _U64, _U64, _U64, _P],
    "bi_mul_u64": [_P, _P, _P, _U32, _U64, _P],
    "bi_mul_u32": [_P, _P, _P, _U32, _U64, _P],
    "bi_mulfull_u64": [_P, _P, _P, _U32, _U64, _P],
    "bi_mulfull_u32": [_P, _P, _P, _U32, _U64, _P],
    "bi_host_mul_u64": [_P, _P, _P, _U32, _U64],
    "bi_host_mul_u32": [_P, _P, _P, _U32, _U64],
    "bi_host_mulfull_u64": [_P, _P, _P, _U32, _U64],
    "bi_host_mulfull_u32": [_P, _P, _P, _U32, _U64],
    "bi_max_limbs_mul_u64": [],
    "bi_max_limbs_mul_u32": [],
    "bi_div_u64": [_P, _P, _P, _P, _P, _U32, _U32, _U64, _P],
    "bi_div_u32": [_P, _P, _P, _P, _P, _U32, _U32, _U64, _P],
    "bi_mul_autotune_u64": [_P, _P, _P, _U32, _U64, _I, _I, _P, _P],
    "bi_mul_autotune_u32": [_P, _P, _P, _U32, _U64, _I, _I, _P, _P],
    "bi_mul_set_tuning_u64": [_U32, _I, _I, _I],
    "bi_mul_set_tuning_u32": [_U32, _I, _I, _I],
    "bi_div_shinv_u64": [_P, _P, _P, _P, _P, _U32, _U32, _U64, _P],
    "bi_div_shinv_u32": [_P, _P, _P, _P, _P, _U32, _U32, _U64, _P],
    "bi_div_long_u64": [_P, _P, _P, _P, _P, _U32, _U32, _U64, _P],
    "bi_div_long_u32": [_P, _P, _P, _P, _P, _U32, _U32, _U64, _P],
    "bi_host_div_u64": [_P, _P, _P, _P, _P, _U32, _U32, _U64],
    "bi_host_div_u32": [_P, _P, _P, _P, _P, _U32, _U32, _U64],
    "bi_max_limbs_div_u64": [],
    "bi_max_limbs_div_u32": [],
    "bi_plan_create": [_P, _P, _U64, _U64, _U64, _U64],
    "bi_plan_execute": [_P, _P, _P, _P, _P],
    "bi_plan_autotune": [_P, _P, _P, _P, _I, _P],
    "bi_plan_set_tuning": [_P, _I, _I, _I],
    "bi_plan_set_mul_word_bits": [_P, _I],
    "bi_plan_get_tuning": [_P, _P],
    "bi_plan_stats": [_P, _P],
    "bi_plan_destroy": [_P],
    "bi_batch_noalloc_max_descs": [],
    "bi_batch_run_noalloc": [_P, _U64, _P, _U64, _P, _U64, _P, _U64, _P],
    "bi_probe_intpipe": [_P, _P],
    "bi_add_chain_u64": [_P, _P, _P, _U32, _U64, _U32, _P],
    "bi_add_chain_u32": [_P, _P, _P, _U32, _U64, _U32, _P],
    "bi_mul_chain_u64": [_P, _P, _P, _U32, _U64, _U32, _P],
    "bi_mul_chain_u32": [_P, _P, _P, _U32, _U64, _U32, _P],
    "bi_cmp_u64": [_P, _P, _P, _U32, _U64, _P],
    "bi_cmp_u32": [_P, _P, _P, _U32, _U64, _P],
    "bi_findk_u64": [_P, _P, _P, _U32, _U64, _P],
    "bi_findk_u32": [_P, _P, _P, _U32, _U64, _P],
    "bi_shift_u64": [_P, _P, ctypes.c_int32, _U32, _U64, _P],
    "bi_shift_u32": [_P, _P, ctypes.c_int32, _U32, _U64, _P],
    "bi_muld_u64": [_P, _P, _P, _U32, _U64, _P],
    "bi_muld_u32": [_P, _P, _P, _U32, _U64, _P],
    "bi_quod_u64": [_P, _P, _P, _P, _U32, _U64, _P],
    "bi_quod_u32": [_P, _P, _P, _P, _U32, _U64, _P],
    "bi_test_add_u64": [_P, _P, _P, _U32],
    "bi_test_add_u32": [_P, _P, _P, _U32],
    "bi_test_sub_u64": [_P, _P, _P, _U32],
    "bi_test_sub_u32": [_P, _P, _P, _U32],
    "bi_test_mul_u64": [_P, _P, _P, _U32],
    "bi_test_mul_u32": [_P, _P, _P, _U32],
    "bi_test_div_u64": [_P, _P, _P, _U32],
    "bi_test_div_u32": [_P, _P, _P, _U32],
    "bi_limbs_from_words": [_P, ctypes.c_size_t, ctypes.c_size_t, _P, _U32],
    "bi_limbs_to_words": [_P, _U32, ctypes.c_size_t, _P, _P],
    "bi_server_create": [_P, _P, _U64, _P, _U64, _U32, _U32, _U32, _U32],
    "bi_server_submit": [_P, _P, _P],
    "bi_server_poll": [_P, _P, _U32, _P],
    "bi_server_release": [_P, _U64],
    "bi_server_inject_dropped": [_P, _P],
    "bi_server_info": [_P, _P],
    "bi_server_destroy": [_P],
    "bi_server_replay": [_P, _P, _P, _U64, _P, _P, _P],
    "bi_serve_replay_plain": [_P, _P, _U64, _P, _P, _U64, _U32, _P, _P, _P],
}
_RESTYPE = {
    "bi_status_string": ctypes.c_char_p,
    "bi_last_error": ctypes.c_char_p,
    "bi_max_limbs_addsub_u64": _U32,
    "bi_max_limbs_addsub_u32": _U32,
    "bi_max_limbs_mul_u64": _U32,
    "bi_max_limbs_mul_u32": _U32,
    "bi_max_limbs_div_u64": _U32,
    "bi_max_limbs_div_u32": _U32,
    "bi_batch_noalloc_max_descs": _U32,
}


def _declare(L: ctypes.CDLL) -> None:
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = _RESTYPE.get(name, _I)


def _check(status: int) -> None:
    if status != 0:
        detail = lib().bi_last_error().decode(errors="replace")
        raise BigIntError(status, detail)


# ---------------------------------------------------------------------------
# device-tensor helpers
# ---------------------------------------------------------------------------

def _wsuffix(t) -> str:
    size = t.element_size()
    if size == 8:
        return "u64"
    if size == 4:
        return "u32"
    raise TypeError("limb tensors must have 4- or 8-byte elements")


def _stream_ptr(stream) -> int:
    import torch

    if stream is None:
        stream = torch.cuda.current_stream()
    return int(stream.cuda_stream)


def _dev2d(t, name: str):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dim() != 2 or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous [n, m] tensor")
    return t


def add(a, b, out=None, stream=None):
    """r = (a + b) mod B^m per row."""
    import torch

    _dev2d(a, "a"), _dev2d(b, "b")
    n, m = a.shape
    if out is None:
        out = torch.empty_like(a)
    w = _wsuffix(a)
    _check(getattr(lib(), f"bi_add_{w}")(a.data_ptr(), b.data_ptr(), out.data_ptr(), m, n, _stream_ptr(stream)))
    return out


def sub(a, b, out=None, sign=None, stream=None):
    """(|a - b|, sign) per row; sign[i] = 1 where a_i < b_i."""
    import torch

    _dev2d(a, "a"), _dev2d(b, "b")
    n, m = a.shape
    if out is None:
        out = torch.empty_like(a)
    if sign is None:
        sign = torch.empty(n, dtype=torch.uint8, device=a.device)
    w = _wsuffix(a)
    _check(getattr(lib(), f"bi_sub_{w}")(a.data_ptr(), b.data_ptr(), out.data_ptr(), sign.data_ptr(),
                                         m, n, _stream_ptr(stream)))
    return out, sign


def mul(a, b, out=None, stream=None):
    """r = (a * b) mod B^m per row (the reference's truncated product)."""
    import torch

    _dev2d(a, "a"), _dev2d(b, "b")
    n, m = a.shape
    if out is None:
        out = torch.empty_like(a)
    _check(getattr(lib(), f"bi_mul_{_wsuffix(a)}")(a.data_ptr(), b.data_ptr(), out.data_ptr(), m, n,
                                                  _stream_ptr(stream)))
    return out


def mulfull(a, b, out=None, stream=None):
    """Full product per row: [n, 2m]."""
    import torch

    _dev2d(a, "a"), _dev2d(b, "b")
    n, m = a.shape
    if out is None:
        out = torch.empty((n, 2 * m), dtype=a.dtype, device=a.device)
    _check(getattr(lib(), f"bi_mulfull_{_wsuffix(a)}")(a.data_ptr(), b.data_ptr(), out.data_ptr(), m, n,
                                                      _stream_ptr(stream)))
    return out


def div(u, v, q=None, r=None, status=None, stream=None, method="auto"):
    """(q, r, status) per row: q = floor(u / v), r = u mod v; status 1 = zero divisor.
    method: "auto" (bi_div_*), "shinv" (the shifted inverse at every size,
    bi_div_shinv_*) or "long" (long division, bi_div_long_*)."""
    import torch

    _dev2d(u, "u"), _dev2d(v, "v")
    n, mu = u.shape
    mv = v.shape[1]
    if q is None:
        q = torch.empty_like(u)
    if r is None:
        r = torch.empty((n, mv), dtype=u.dtype, device=u.device)
    if status is None:
        status = torch.empty(n, dtype=torch.uint8, device=u.device)
    if method not in ("auto", "shinv", "long"):
        raise ValueError(f"div: unknown method {method!r}")
    name = f"bi_div_{_wsuffix(u)}" if method == "auto" else f"bi_div_{method}_{_wsuffix(u)}"
    _check(getattr(lib(), name)(u.data_ptr(), v.data_ptr(), q.data_ptr(), r.data_ptr(),
                                status.data_ptr(), mu, mv, n, _stream_ptr(stream)))
    return q, r, status


def mul_autotune(a, b, r=None, full: bool = True, reps: int = 3, stream=None):
    """Time the CTA multiply's tilings on (a, b) -- and the 32-bit-word warp
    kernel for full products of at most 32 64-bit limbs, the one-thread-an-
    instance kernel for full products of at most 24 and truncated ones of at
    most 32 -- and keep the fastest for this (limb
    width, full, m); returns (instances per CTA, slices), (0, 0) when the warp
    kernel was fastest, (0, 1) for the thread kernel.  r receives the product
    as mulfull/mul write it."""
    import torch

    _dev2d(a, "a"), _dev2d(b, "b")
    n, m = a.shape
    if r is None:
        r = torch.empty((n, 2 * m if full else m), dtype=a.dtype, device=a.device)
    chosen = (ctypes.c_int * 2)()
    _check(getattr(lib(), f"bi_mul_autotune_{_wsuffix(a)}")(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n,
                                                           1 if full else 0, reps, ctypes.cast(chosen, ctypes.c_void_p),
                                                           _stream_ptr(stream)))
    return int(chosen[0]), int(chosen[1])


def mul_set_tuning(m: int, dtype, full: bool, ipc: int, slices: int = 1):
    """Set the CTA multiply's tiling for (limb width, full, m) by hand; ipc=-1
    picks a per-instance kernel (slices 0: the warp kernel, full products
    only; 1: the thread kernel); ipc=0 returns to the library's own choice."""
    w = "u64" if np.dtype(dtype).itemsize == 8 else "u32"
    _check(getattr(lib(), f"bi_mul_set_tuning_{w}")(m, 1 if full else 0, ipc, slices))


def add_chain(a, b, p: int, out=None, stream=None):
    """r1 = a + b, then p-1 times r = r1 + r: p (a + b) mod B^m per row."""
    _dev2d(a, "a")
    _dev2d(b, "b")
    n, m = a.shape
    r = out if out is not None else a.new_empty(a.shape)
    _check(getattr(lib(), f"bi_add_chain_{_wsuffix(a)}")(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, p,
                                                         _stream_ptr(stream)))
    return r


def mul_chain(a, b, p: int, out=None, stream=None):
    """r1 = a * b, then p-1 times r = r1 * r, truncated: (a b)^p mod B^m per row."""
    _dev2d(a, "a")
    _dev2d(b, "b")
    n, m = a.shape
    r = out if out is not None else a.new_empty(a.shape)
    _check(getattr(lib(), f"bi_mul_chain_{_wsuffix(a)}")(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, p,
                                                         _stream_ptr(stream)))
    return r


# ---------------------------------------------------------------------------
# the division prototype's helper primitives, batched (bi_cmp, bi_findk, ...)
# ---------------------------------------------------------------------------

def cmp(a, b, stream=None):
    """int8 per row: -1, 0, 1 as a <, ==, > b."""
    import torch

    _dev2d(a, "a")
    _dev2d(b, "b")
    n, m = a.shape
    out = torch.empty(n, dtype=torch.int8, device=a.device)
    _check(getattr(lib(), f"bi_cmp_{_wsuffix(a)}")(a.data_ptr(), b.data_ptr(), out.data_ptr(), m, n,
                                                   _stream_ptr(stream)))
    return out


def findk(a, stream=None):
    """(k, zero): index of each row's top nonzero limb (0 for zero), and a == 0."""
    import torch

    _dev2d(a, "a")
    n, m = a.shape
    k = torch.empty(n, dtype=torch.int32, device=a.device)
    z = torch.empty(n, dtype=torch.uint8, device=a.device)
    _check(getattr(lib(), f"bi_findk_{_wsuffix(a)}")(a.data_ptr(), k.data_ptr(), z.data_ptr(), m, n,
                                                     _stream_ptr(stream)))
    return k, z


def shift(a, digits: int, stream=None):
    """Shift each row by whole limbs: up (multiply by B^digits) for digits >= 0."""
    _dev2d(a, "a")
    n, m = a.shape
    r = a.new_empty(a.shape)
    _check(getattr(lib(), f"bi_shift_{_wsuffix(a)}")(a.data_ptr(), r.data_ptr(), digits, m, n,
                                                     _stream_ptr(stream)))
    return r


def muld(a, d, stream=None):
    """r = a * d mod B^m per row, d one limb per row (a tensor of n limbs)."""
    _dev2d(a, "a")
    n, m = a.shape
    r = a.new_empty(a.shape)
    _check(getattr(lib(), f"bi_muld_{_wsuffix(a)}")(a.data_ptr(), d.data_ptr(), r.data_ptr(), m, n,
                                                    _stream_ptr(stream)))
    return r


def quod(a, d, stream=None):
    """(q, rem): floor(a / d) and a mod d per row, d one limb per row."""
    _dev2d(a, "a")
    n, m = a.shape
    q = a.new_empty(a.shape)
    rem = d.new_empty(d.shape)
    _check(getattr(lib(), f"bi_quod_{_wsuffix(a)}")(a.data_ptr(), d.data_ptr(), q.data_ptr(), rem.data_ptr(), m, n,
                                                    _stream_ptr(stream)))
    return q, rem


def limbs_from_words(words: np.ndarray, m: int) -> np.ndarray:
    """m u64 limbs from a word array in GMP's order -1 (mpz_export(..., -1, size, 0, 0, ...))."""
    words = np.ascontiguousarray(words)
    out = np.zeros(m, dtype=np.uint64)
    _check(lib().bi_limbs_from_words(words.ctypes.data_as(ctypes.c_void_p), words.size, words.itemsize,
                                     out.ctypes.data_as(ctypes.c_void_p), m))
    return out


def limbs_to_words(limbs: np.ndarray, dtype=np.uint32) -> np.ndarray:
    """Words of `dtype` in GMP's order -1 without leading zeros (what mpz_export writes)."""
    limbs = np.ascontiguousarray(limbs, dtype=np.uint64)
    size = np.dtype(dtype).itemsize
    out = np.zeros(limbs.size * 8 // size, dtype=dtype)
    cnt = ctypes.c_size_t()
    _check(lib().bi_limbs_to_words(limbs.ctypes.data_as(ctypes.c_void_p), limbs.size, size,
                                   out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(cnt)))
    return out[: cnt.value]


def fill_splitmix64(t, seed: int, offset: int = 0, stream=None):
    """Fill an 8-byte-element CUDA tensor with the splitmix64 stream ``seed``."""
    if not t.is_cuda or t.element_size() != 8 or not t.is_contiguous():
        raise ValueError("fill_splitmix64 needs a contiguous CUDA tensor of 8-byte elements")
    _check(lib().bi_fill_splitmix64(t.data_ptr(), t.numel(), seed & (2**64 - 1), offset, _stream_ptr(stream)))
    return t


PROBE_FORMS = ("mad.lo.u32", "mad.hi.u32", "mad.wide.u32", "mad.cc carry-chain rows", "mul.lo/hi.u64",
               "mad.wide.u32 column sums")


def probe_intpipe(stream=None) -> dict:
    """Measured 32x32-bit word products per second for each instruction form."""
    rates = (ctypes.c_double * 6)()
    _check(lib().bi_probe_intpipe(ctypes.cast(rates, ctypes.c_void_p), _stream_ptr(stream)))
    return dict(zip(PROBE_FORMS, list(rates)))


# ---------------------------------------------------------------------------
# uneven batches (include/bigint_gb300.h: bi_desc, bi_plan_*)
# ---------------------------------------------------------------------------

OP_ADD, OP_SUB, OP_MUL, OP_MULFULL, OP_DIV = 0, 1, 2, 3, 4

DESC_DTYPE = np.dtype([("op", "<u4"), ("m", "<u4"), ("mb", "<u4"), ("width", "<u4"),
                       ("a", "<u8"), ("b", "<u8"), ("r", "<u8"), ("r2", "<u8"), ("flag", "<u8")])


class Plan:
    """A bucketed, graph-captured execution plan for an uneven batch.

    in_limbs, out_limbs and nflags are the sizes of the input arena, the
    output arena (64-bit limbs) and the flag arena (bytes) the plan will run
    on; every descriptor is checked against them when the plan is built
    (nflags = 0: the plan writes no flags and execute takes flags=None)."""

    def __init__(self, descs: np.ndarray, in_limbs: int, out_limbs: int, nflags: int = 0):
        descs = np.ascontiguousarray(descs, dtype=DESC_DTYPE)
        self.count = len(descs)
        self._h = ctypes.c_void_p()
        _check(lib().bi_plan_create(ctypes.byref(self._h), descs.ctypes.data_as(ctypes.c_void_p), self.count,
                                    int(in_limbs), int(out_limbs), int(nflags)))

    def execute(self, arena_in, arena_out, flags=None, stream=None):
        _check(lib().bi_plan_execute(self._h, arena_in.data_ptr(), arena_out.data_ptr(),
                                     flags.data_ptr() if flags is not None else None, _stream_ptr(stream)))

    def autotune(self, arena_in, arena_out, flags=None, reps: int = 3):
        chosen = (ctypes.c_int * 3)()
        _check(lib().bi_plan_autotune(self._h, arena_in.data_ptr(), arena_out.data_ptr(),
                                      flags.data_ptr() if flags is not None else None, reps,
                                      ctypes.cast(chosen, ctypes.c_void_p)))
        return self.tuning()

    def set_tuning(self, rows: int, vec: int, ipc_div: int):
        _check(lib().bi_plan_set_tuning(self._h, rows, vec, ipc_div))

    def set_mul_word_bits(self, bits: int):
        """Word width of the arithmetic for full products of at most 32
        limbs: 32 (the warp kernel) or 64 (the CTA kernel)."""
        _check(lib().bi_plan_set_mul_word_bits(self._h, bits))

    def tuning(self) -> dict:
        t = (ctypes.c_int * 4)()
        _check(lib().bi_plan_get_tuning(self._h, ctypes.cast(t, ctypes.c_void_p)))
        return {"addsub_rows": t[0], "addsub_limbs_per_lane_row": t[1], "mul_ipc_divisor": t[2],
                "mul_small_word_bits": t[3]}

    def stats(self) -> dict:
        st = (ctypes.c_uint64 * 6)()
        _check(lib().bi_plan_stats(self._h, ctypes.cast(st, ctypes.c_void_p)))
        keys = ("addsub", "mul", "mul_items", "div", "mul_smem_bytes", "div_smem_bytes")
        return dict(zip(keys, list(st)))

    def close(self):
        if self._h:
            lib().bi_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# serving loop (include/bigint_gb300.h: bi_server_*)
# ---------------------------------------------------------------------------

BI_EBUSY = 7

COMPLETION_DTYPE = np.dtype([("ticket", "<u8"), ("r", "<u8"), ("r2", "<u8"), ("status", "<u4"), ("op", "<u4")])
REPORT_KEYS = ("requests", "launches", "busy", "duration_s", "offered_rps", "achieved_rps",
               "p50_us", "p90_us", "p99_us", "p999_us", "max_us", "mean_us")


def _report(buf) -> dict:
    return dict(zip(REPORT_KEYS, [float(x) for x in buf]))


class Server:
    """A device-resident request loop over the operand arena `operands`
    (a uint64 CUDA tensor).  `arena` (a uint64 CUDA tensor) receives the
    results; its size is the server's memory budget for results in flight."""

    def __init__(self, operands, arena, ring_slots: int = 0, max_limbs: int = 0, ctas: int = 0,
                 idle_us: int = 0):
        self.operands, self.arena = operands, arena
        self._h = ctypes.c_void_p()
        _check(lib().bi_server_create(ctypes.byref(self._h), operands.data_ptr(), operands.numel(),
                                      arena.data_ptr(), arena.numel(), ring_slots, max_limbs, ctas, idle_us))

    def submit(self, desc):
        """Ticket of the admitted request, or None if the server is full."""
        d = np.ascontiguousarray(np.asarray(desc, dtype=DESC_DTYPE).reshape(1))
        t = ctypes.c_uint64()
        st = lib().bi_server_submit(self._h, d.ctypes.data_as(ctypes.c_void_p), ctypes.byref(t))
        if st == BI_EBUSY:
            return None
        _check(st)
        return t.value

    def poll(self, max_count: int = 4096) -> np.ndarray:
        out = np.zeros(max_count, dtype=COMPLETION_DTYPE)
        k = ctypes.c_uint32()
        _check(lib().bi_server_poll(self._h, out.ctypes.data_as(ctypes.c_void_p), max_count, ctypes.byref(k)))
        return out[: k.value]

    def release(self, ticket: int):
        _check(lib().bi_server_release(self._h, int(ticket)))

    def inject_dropped(self):
        """Publish a slot whose contents never arrive (failure injection);
        returns its ticket, which completes with status 255."""
        t = ctypes.c_uint64()
        _check(lib().bi_server_inject_dropped(self._h, ctypes.byref(t)))
        return t.value

    def info(self) -> dict:
        v = (ctypes.c_uint64 * 10)()
        _check(lib().bi_server_info(self._h, ctypes.cast(v, ctypes.c_void_p)))
        keys = ("arena_ptr", "arena_limbs", "ctas", "smem_bytes", "launches", "busy", "lost", "ring_slots",
                "submitted", "completed")
        return dict(zip(keys, list(v)))

    def replay(self, descs: np.ndarray, arrival_ns: np.ndarray):
        """Open-loop replay; returns (latency_ns, completions, report)."""
        descs = np.ascontiguousarray(descs, dtype=DESC_DTYPE)
        arrival_ns = np.ascontiguousarray(arrival_ns, dtype=np.uint64)
        n = len(descs)
        lat = np.zeros(n, np.uint64)
        done = np.zeros(n, COMPLETION_DTYPE)
        rep = (ctypes.c_double * len(REPORT_KEYS))()
        _check(lib().bi_server_replay(self._h, descs.ctypes.data_as(ctypes.c_void_p),
                                      arrival_ns.ctypes.data_as(ctypes.c_void_p), n,
                                      lat.ctypes.data_as(ctypes.c_void_p), done.ctypes.data_as(ctypes.c_void_p),
                                      ctypes.cast(rep, ctypes.c_void_p)))
        return lat, done, _report(rep)

    def close(self):
        if self._h:
            lib().bi_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def replay_plain(operands, arena, descs: np.ndarray, arrival_ns: np.ndarray, streams: int = 1):
    """The same open-loop stream with one library launch per request;
    returns (latency_ns, completions, report)."""
    descs = np.ascontiguousarray(descs, dtype=DESC_DTYPE)
    arrival_ns = np.ascontiguousarray(arrival_ns, dtype=np.uint64)
    n = len(descs)
    lat = np.zeros(n, np.uint64)
    done = np.zeros(n, COMPLETION_DTYPE)
    rep = (ctypes.c_double * len(REPORT_KEYS))()
    _check(lib().bi_serve_replay_plain(operands.data_ptr(), arena.data_ptr(), arena.numel(),
                                       descs.ctypes.data_as(ctypes.c_void_p),
                                       arrival_ns.ctypes.data_as(ctypes.c_void_p), n, streams,
                                       lat.ctypes.data_as(ctypes.c_void_p), done.ctypes.data_as(ctypes.c_void_p),
                                       ctypes.cast(rep, ctypes.c_void_p)))
    return lat, done, _report(rep)


# ---------------------------------------------------------------------------
# host (numpy) entry points: the reference's synchronous wrapper shape
# ---------------------------------------------------------------------------

def _np_w(a: np.ndarray) -> str:
    if a.dtype == np.uint64:
        return "u64"
    if a.dtype == np.uint32:
        return "u32"
    raise TypeError("limb arrays must be uint32 or uint64")


def _nptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def host_add(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    n, m = a.shape
    r = np.empty_like(a)
    _check(getattr(lib(), f"bi_host_add_{_np_w(a)}")(_nptr(a), _nptr(b), _nptr(r), m, n))
    return r


def host_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    n, m = a.shape
    r = np.empty_like(a)
    _check(getattr(lib(), f"bi_host_mul_{_np_w(a)}")(_nptr(a), _nptr(b), _nptr(r), m, n))
    return r


def host_mulfull(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    n, m = a.shape
    r = np.empty((n, 2 * m), dtype=a.dtype)
    _check(getattr(lib(), f"bi_host_mulfull_{_np_w(a)}")(_nptr(a), _nptr(b), _nptr(r), m, n))
    return r


def host_div(u: np.ndarray, v: np.ndarray):
    """(q, r, status); raises BigIntError(BI_EDIV0) if any divisor is zero."""
    u, v = np.ascontiguousarray(u), np.ascontiguousarray(v)
    n, mu = u.shape
    mv = v.shape[1]
    q = np.empty_like(u)
    r = np.empty((n, mv), dtype=u.dtype)
    st = np.zeros(n, dtype=np.uint8)
    _check(getattr(lib(), f"bi_host_div_{_np_w(u)}")(_nptr(u), _nptr(v), _nptr(q), _nptr(r), _nptr(st), mu, mv, n))
    return q, r, st


def host_sub(a: np.ndarray, b: np.ndarray):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    n, m = a.shape
    r = np.empty_like(a)
    s = np.empty(n, dtype=np.uint8)
    _check(getattr(lib(), f"bi_host_sub_{_np_w(a)}")(_nptr(a), _nptr(b), _nptr(r), _nptr(s), m, n))
    return r, s


# ---------------------------------------------------------------------------
# numpy <-> torch bit-preserving transfers (torch has no full uint64 support)
# ---------------------------------------------------------------------------

def to_device(x: np.ndarray, device="cuda"):
    import torch

    x = np.ascontiguousarray(x)
    view = {8: np.int64, 4: np.int32, 1: np.uint8}[x.dtype.itemsize]
    return torch.from_numpy(x.view(view)).to(device)


def to_host(t, dtype) -> np.ndarray:
    return t.cpu().numpy().view(dtype)
