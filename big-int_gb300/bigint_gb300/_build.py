"""Build recipe for libbigint_gb300.so (sm_103a only).

Compiles every ``csrc/*.cu`` translation unit with nvcc in parallel and links
them into ``bigint_gb300/libbigint_gb300.so`` inside the source tree.  Object
files go to ``big-int_gb300/_build/`` (git-ignored).  A unit is recompiled
when it or any header under ``csrc/`` or ``include/`` is newer than its
object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
PROJ_DIR = os.path.dirname(PKG_DIR)                 # big-int_gb300/
REPO_DIR = os.path.dirname(PROJ_DIR)
CSRC = os.path.join(PROJ_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
OBJ_DIR = os.path.join(PROJ_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libbigint_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC,-O2,-Wall", "-I", INCLUDE, "-I", CSRC,
    ]


def _newest_header() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    hs += glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src: str, obj: str, extra: list[str]) -> tuple[str, int, str]:
    cmd = [_nvcc()] + _flags() + extra + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    return src, p.returncode, p.stdout + p.stderr


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile the CUDA sources and link the shared library; return its path."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_t = _newest_header()
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(OBJ_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_t):
            jobs.append((s, o))
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda j: _compile(j[0], j[1], extra), jobs))
        failed = [r for r in results if r[1] != 0]
        for src, rc, out in results:
            if verbose or ptxas_info or rc != 0:
                print(f"== {os.path.basename(src)} (rc={rc})\n{out}")
        if failed:
            raise RuntimeError("nvcc failed for: " + ", ".join(os.path.basename(f[0]) for f in failed))
    lib_t = os.path.getmtime(LIB_PATH) if os.path.exists(LIB_PATH) else -1.0
    if jobs or force or lib_t < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB_PATH] + objs + ["-lcudart", "-lcuda"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n" + p.stdout + p.stderr)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
