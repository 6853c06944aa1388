"""CPU tests of the C ABI boundary: the library builds for sm_103a, loads,
exports every function include/*.h declares, and validates arguments before
it touches a GPU (no compute call is made here)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for mt in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(bi_\w+)\s*\(", src, flags=re.M):
            names.add(mt.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def L():
    import bigint_gb300 as B

    B.build()
    return B.lib()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("bi_add_u64", "bi_sub_u64", "bi_host_add_u64", "bi_status_string"):
        assert must in names


def test_every_declared_symbol_is_exported(L):
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_python_signatures_cover_header(L):
    import bigint_gb300 as B

    missing = [n for n in declared_functions() if n not in B.SIGNATURES]
    assert not missing, missing


def test_status_strings(L):
    assert L.bi_status_string(0) == b"BI_OK"
    assert L.bi_status_string(2) == b"BI_EDIV0"
    assert L.bi_version() >= 100


def test_zero_instances_is_noop(L):
    p = ctypes.c_void_p(0)
    assert L.bi_add_u64(p, p, p, 4, 0, None) == 0
    assert L.bi_sub_u32(p, p, p, p, 4, 0, None) == 0


def test_invalid_arguments_rejected_before_launch(L):
    fake = ctypes.c_void_p(0x1000)          # never dereferenced: validation fails first
    assert L.bi_add_u64(fake, fake, fake, 0, 5, None) == 1          # m == 0
    assert L.bi_add_u64(None, fake, fake, 4, 5, None) == 1         # NULL
    assert L.bi_add_u64(ctypes.c_void_p(0x1004), fake, fake, 4, 5, None) == 1  # misaligned
    assert b"aligned" in L.bi_last_error()
    big = L.bi_max_limbs_addsub_u64() + 2
    assert L.bi_add_u64(fake, fake, fake, big, 1, None) == 6         # unsupported size


def test_mul_tuning_arguments_checked_on_host(L):
    assert L.bi_mul_set_tuning_u64(0, 1, 4, 1) == 1                  # m == 0
    assert L.bi_mul_set_tuning_u64(64, 1, 4, 3) == 1                 # slices not a power of two
    assert L.bi_mul_set_tuning_u64(64, 1, 4096, 1) == 1              # more instances than a CTA holds
    assert L.bi_mul_set_tuning_u64(64, 1, -1, 1) == 1                # no per-instance kernel at 64 limbs
    assert L.bi_mul_set_tuning_u64(25, 1, -1, 1) == 1                # thread kernel: full products up to 24 limbs
    assert L.bi_mul_set_tuning_u64(33, 0, -1, 1) == 1                # and truncated ones up to 32
    assert L.bi_mul_set_tuning_u64(8, 1, -1, 2) == 1                 # no such per-instance kernel
    assert L.bi_mul_set_tuning_u64(8, 0, -1, 0) == 1                 # truncated products: no warp kernel
    assert L.bi_mul_set_tuning_u64(8, 1, -2, 1) == 1
    assert L.bi_mul_set_tuning_u64(1 << 20, 1, 1, 1) == 6            # unsupported size
    fake = ctypes.c_void_p(0x1000)
    assert L.bi_mul_autotune_u64(fake, fake, fake, 64, 0, 1, 3, None, None) == 1   # n == 0
    assert L.bi_mul_autotune_u64(fake, fake, fake, 64, 8, 1, 0, None, None) == 1   # reps == 0
    assert L.bi_mul_autotune_u64(None, fake, fake, 64, 8, 1, 3, None, None) == 1   # NULL


def test_library_built_for_sm103a():
    import bigint_gb300 as B

    assert "arch=compute_103a,code=sm_103a" in " ".join(B._build.ARCH)
    assert os.path.exists(B.LIB_PATH)


def test_server_rejects_bad_arguments_on_host(L):
    """The serving loop validates its arguments before any CUDA call."""
    h = ctypes.c_void_p()
    fake = ctypes.c_void_p(0x1000)
    assert L.bi_server_create(ctypes.byref(h), None, 0, None, 0, 0, 0, 0, 0) == 1      # no operands
    assert L.bi_server_create(None, fake, 16, None, 0, 0, 0, 0, 0) == 1                 # NULL handle
    assert L.bi_server_create(ctypes.byref(h), ctypes.c_void_p(0x1008), 16, None, 0, 0, 0, 0, 0) == 1  # misaligned
    assert L.bi_server_create(ctypes.byref(h), fake, 16, None, 0, 3, 0, 0, 0) == 1      # ring not a power of 2
    assert L.bi_server_create(ctypes.byref(h), fake, 16, None, 0, 0, 4096, 0, 0) == 6   # max_limbs too large
    assert not h.value
    assert L.bi_server_submit(None, None, None) == 1
    assert L.bi_server_poll(None, None, 0, None) == 1
    assert L.bi_server_destroy(None) == 0
    assert L.bi_status_string(7) == b"BI_EBUSY"


def test_gmp_word_converters_round_trip(L):
    """bi_limbs_from_words / bi_limbs_to_words against Python integers: GMP's
    order -1 word arrays of 1, 2, 4 and 8 bytes (host code, no GPU)."""
    import numpy as np

    import bigint_gb300 as B

    rng = np.random.default_rng(5)
    for dt in (np.uint8, np.uint16, np.uint32, np.uint64):
        for nbits in (0, 1, 63, 64, 65, 1000, 4096):
            x = int(rng.integers(0, 2**62)) ** 80 % (1 << nbits) if nbits else 0
            size = np.dtype(dt).itemsize
            nw = max(1, (nbits + 8 * size - 1) // (8 * size))
            words = np.array([(x >> (8 * size * k)) & ((1 << (8 * size)) - 1) for k in range(nw)], dtype=dt)
            m = max(1, (nbits + 63) // 64)
            limbs = B.limbs_from_words(words, m)
            assert sum(int(v) << (64 * j) for j, v in enumerate(limbs)) == x
            back = B.limbs_to_words(limbs, dt)
            assert sum(int(v) << (8 * size * k) for k, v in enumerate(back)) == x
            assert len(back) == 0 if x == 0 else back[-1] != 0        # no leading zero words
    with pytest.raises(B.BigIntError):
        B.limbs_from_words(np.array([1, 2, 3], dtype=np.uint64), 2)   # needs 3 limbs


def test_plan_tuning_arguments_checked_on_host(L):
    t = (ctypes.c_int * 4)()
    assert L.bi_plan_set_mul_word_bits(None, 32) == 1                 # NULL plan
    assert L.bi_plan_get_tuning(None, ctypes.cast(t, ctypes.c_void_p)) == 1
    assert L.bi_plan_set_tuning(None, 4, 2, 1) == 1
    assert L.bi_plan_autotune(None, None, None, None, 1, None) == 1


def _desc(B, op, m, mb, a, b, r, r2=0, flag=0):
    d = np.zeros(1, dtype=B.DESC_DTYPE)
    d[0]["op"], d[0]["m"], d[0]["mb"] = op, m, mb
    d[0]["a"], d[0]["b"], d[0]["r"], d[0]["r2"], d[0]["flag"] = a, b, r, r2, flag
    return d


def test_batch_descriptors_checked_against_arenas_on_host(L):
    """Every operand, result and flag a batch descriptor names must lie inside
    its arena: out-of-range offsets for each op are refused with BI_EINVAL by
    bi_plan_create and bi_batch_run_noalloc before any device work (the
    arena pointers below are never dereferenced)."""
    import bigint_gb300 as B

    IN, OUT, NF = 1000, 1000, 10
    cases = []
    for op in (B.OP_ADD, B.OP_SUB, B.OP_MUL, B.OP_MULFULL, B.OP_DIV):
        m, mb = 40, (20 if op == B.OP_DIV else 40)
        lr = 2 * m if op == B.OP_MULFULL else m
        cases += [
            _desc(B, op, m, mb, IN - m + 1, 0, 0, 500, 0),           # a runs past the input arena
            _desc(B, op, m, mb, 0, IN - mb + 1, 0, 500, 0),          # b runs past it
            _desc(B, op, m, mb, 0, 100, OUT - lr + 1, 0, 0),         # r runs past the output arena
            _desc(B, op, m, mb, 0, 100, 2 ** 64 - 8, 500, 0),        # an offset that wraps
        ]
        if op == B.OP_DIV:
            cases.append(_desc(B, op, m, mb, 0, 100, 0, OUT - mb + 1, 0))   # r2 runs past it
        if op in (B.OP_SUB, B.OP_DIV):
            cases.append(_desc(B, op, m, mb, 0, 100, 0, 500, NF))          # flag past the flag arena
    fake = ctypes.c_void_p(4096)                                      # 16-byte aligned, never read
    for d in cases:
        h = ctypes.c_void_p()
        st = L.bi_plan_create(ctypes.byref(h), d.ctypes.data_as(ctypes.c_void_p), 1, IN, OUT, NF)
        assert st == 1 and not h.value, (d, L.bi_last_error())
        assert b"outside" in L.bi_last_error()
        st = L.bi_batch_run_noalloc(d.ctypes.data_as(ctypes.c_void_p), 1, fake, IN, fake, OUT, fake, NF, None)
        assert st == 1 and b"outside" in L.bi_last_error(), (d, L.bi_last_error())
    # flags without a flag arena
    d = _desc(B, B.OP_ADD, 4, 4, 0, 4, 0)
    st = L.bi_batch_run_noalloc(d.ctypes.data_as(ctypes.c_void_p), 1, fake, IN, fake, OUT, fake, 0, None)
    assert st == 1 and b"nflags" in L.bi_last_error()
