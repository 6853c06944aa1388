"""Loader for the reference's own CUDA kernels (baseline/_ref/libref_gpu.so).

The shared library is built from baseline/ref_gpu.cu and the reference's
kernel headers staged by install_ref.sh.  It is a baseline to measure
against and to check parity with -- never part of the library's data path.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
HDR = os.path.join(REF_DIR, "cuda", "ker-mul.cu.h")
LIB = os.path.join(REF_DIR, "libref_gpu.so")
SRC = os.path.join(HERE, "ref_gpu.cu")

_lib = None


def reference_checkout():
    """The reference checkout: $BIGINT_REF, else a `reference` directory
    beside the repository; None when neither exists (as on a GPU machine)."""
    for cand in (os.environ.get("BIGINT_REF"), os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")):
        if cand and os.path.isdir(cand):
            return cand
    return None


def build() -> bool:
    """Stage the reference headers (when the checkout exists) and compile."""
    ref = reference_checkout()
    if ref:
        subprocess.run(["sh", os.path.join(HERE, "install_ref.sh")], capture_output=True,
                       env=dict(os.environ, REF=ref))
    if not os.path.exists(HDR):
        return False
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        return True
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-shared", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w",
           "-I", os.path.dirname(HDR), SRC, "-o", LIB]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("reference kernel build failed:\n" + p.stdout + p.stderr)
    return True


def lib():
    """The reference-kernel library, or None if it is not available."""
    global _lib
    if _lib is None and os.path.exists(LIB):
        L = ctypes.CDLL(LIB)
        for name in ("ref_add_u64", "ref_mul_u64", "ref_mul_u32", "ref_add10_u64", "ref_add10v1_u64", "ref_mul6_u64"):
            f = getattr(L, name)
            f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
            f.restype = ctypes.c_int
        _lib = L
    return _lib


ADD_SIZES = [16, 32, 64, 128, 256, 512, 1024, 2048, 4096]   # u64 limbs
MUL_SIZES_U64 = [16, 32, 64, 128, 256, 512, 1024, 2048]   # the reference's own sweep reaches 16 (cuda/main.cu:501-512)
MUL_SIZES_U32 = [16, 32, 64, 128]
ADD10_SIZES = [16, 128, 1024, 4096]   # u64 limbs (baddKer3Bench<..., 10>)
ADD10_V1_SIZES = [16, 128, 1024]      # baddKer1Bench<..., 10> (one instance per block, m <= 1024)
MUL6_SIZES = [64, 256, 1024]          # u64 limbs (convMul5Bench<..., 6>)
