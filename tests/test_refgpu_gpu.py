"""Parity with the reference's own CUDA kernels on the same seeded inputs:
baddKer3 (C-V3 add) and convMul5 (C-V5 truncated multiply, and the full
product through zero-padded 2m-limb inputs), compiled unmodified for sm_103a
from the staged reference headers.  Skipped where those headers were not
staged (the reference checkout was absent when the repository was built)."""
import os
import sys

import numpy as np
import pytest

from bigint_gb300.workloads import uniform_limbs

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "baseline"))


@pytest.fixture(scope="module")
def ref():
    import refgpu

    if not refgpu.build() or refgpu.lib() is None:
        pytest.skip("reference CUDA kernels not staged")
    return refgpu


def _sp():
    import torch

    return int(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("m", [16, 64, 256, 1024, 4096])
def test_add_matches_reference_kernel(bigint, ref, m):
    import torch

    B = bigint
    n = max(256, 65536 // m)
    a = uniform_limbs(900 + m, n, m)
    b = uniform_limbs(901 + m, n, m)
    a[0] = np.iinfo(np.uint64).max
    b[0] = 0
    b[0, 0] = 1
    da, db = B.to_device(a), B.to_device(b)
    rr = torch.empty_like(da)
    assert ref.lib().ref_add_u64(da.data_ptr(), db.data_ptr(), rr.data_ptr(), m, n, _sp()) == 0
    ours = B.add(da, db)
    assert bool((ours == rr).all())


@pytest.mark.parametrize("m", [16, 32, 64, 256, 1024])
def test_mul_matches_reference_kernel(bigint, ref, m):
    import torch

    B = bigint
    n = 512
    a = uniform_limbs(910 + m, n, m)
    b = uniform_limbs(911 + m, n, m)
    da, db = B.to_device(a), B.to_device(b)
    # truncated product: convMul5 at size m
    rr = torch.empty_like(da)
    assert ref.lib().ref_mul_u64(da.data_ptr(), db.data_ptr(), rr.data_ptr(), m, n, _sp()) == 0
    assert bool((B.mul(da, db) == rr).all())
    # full product: convMul5 at size 2m on zero-padded inputs
    pa = torch.zeros((n, 2 * m), dtype=torch.int64, device="cuda")
    pb = torch.zeros_like(pa)
    pa[:, :m] = da
    pb[:, :m] = db
    rf = torch.empty_like(pa)
    assert ref.lib().ref_mul_u64(pa.data_ptr(), pb.data_ptr(), rf.data_ptr(), 2 * m, n, _sp()) == 0
    assert bool((B.mulfull(da, db) == rf).all())


@pytest.mark.parametrize("m", [16, 32])
def test_small_u32_mul_matches_reference_kernel(bigint, ref, m):
    """u32 words at the small end of the reference's own multiply sweep: the
    truncated product against convMul5 at m, the full one against convMul5 at
    2m on zero-padded inputs (the thread and warp kernels here)."""
    import torch

    B = bigint
    n = 512
    a = uniform_limbs(930 + m, n, m, np.uint32)
    b = uniform_limbs(931 + m, n, m, np.uint32)
    a[0] = np.iinfo(np.uint32).max
    b[0] = np.iinfo(np.uint32).max
    da, db = B.to_device(a), B.to_device(b)
    rr = torch.empty_like(da)
    assert ref.lib().ref_mul_u32(da.data_ptr(), db.data_ptr(), rr.data_ptr(), m, n, _sp()) == 0
    assert bool((B.mul(da, db) == rr).all())
    pa = torch.zeros((n, 2 * m), dtype=torch.int32, device="cuda")
    pb = torch.zeros_like(pa)
    pa[:, :m] = da
    pb[:, :m] = db
    rf = torch.empty_like(pa)
    assert ref.lib().ref_mul_u32(pa.data_ptr(), pb.data_ptr(), rf.data_ptr(), 2 * m, n, _sp()) == 0
    assert bool((B.mulfull(da, db) == rf).all())


def test_mul2048_u32_matches_reference_kernel(bigint, ref):
    import torch

    from bigint_gb300.workloads import mul2048_u32

    B = bigint
    a, b = mul2048_u32()
    n, m = a.shape
    pa = np.zeros((n, 2 * m), np.uint32)
    pb = np.zeros((n, 2 * m), np.uint32)
    pa[:, :m] = a
    pb[:, :m] = b
    da, db = B.to_device(pa), B.to_device(pb)
    rf = torch.empty_like(da)
    assert ref.lib().ref_mul_u32(da.data_ptr(), db.data_ptr(), rf.data_ptr(), 2 * m, n, _sp()) == 0
    ours = B.mulfull(B.to_device(a), B.to_device(b))
    assert bool((ours == rf).all())


@pytest.mark.parametrize("m", [16, 128, 1024])
def test_add_chain_matches_reference_ten_additions(bigint, ref, m):
    """bi_add_chain with p = 10 against baddKer1Bench<U64bits, m, 10>, whose
    result is the thesis's 10(u+v)."""
    import torch

    B = bigint
    n = max(256, 65536 // m)
    a = uniform_limbs(920 + m, n, m)
    b = uniform_limbs(921 + m, n, m)
    a[0] = np.iinfo(np.uint64).max
    b[0] = 0
    b[0, 0] = 1
    da, db = B.to_device(a), B.to_device(b)
    rr = torch.empty_like(da)
    assert ref.lib().ref_add10v1_u64(da.data_ptr(), db.data_ptr(), rr.data_ptr(), m, n, _sp()) == 0
    assert bool((B.add_chain(da, db, 10) == rr).all())


def test_reference_v3_ten_additions_drops_carries(bigint, ref, oracle):
    """baddKer3Bench adds into the buffer it reads (ker-add.cu.h:283-291), so
    from the second step on it compares each new limb with itself and loses
    every carry: steps 2..10 double each limb on its own.  Documented here
    on an input whose first sum has a limb with its top bit set."""
    import torch

    B = bigint
    m, n = 16, 256
    a = uniform_limbs(940, n, m)
    b = uniform_limbs(941, n, m)
    da, db = B.to_device(a), B.to_device(b)
    rr = torch.empty_like(da)
    assert ref.lib().ref_add10_u64(da.data_ptr(), db.data_ptr(), rr.data_ptr(), m, n, _sp()) == 0
    got = B.to_host(rr, np.uint64)
    r1 = oracle.add(a, b)
    limbwise = (r1 << np.uint64(9))            # each limb doubled nine times, no carries
    assert (got == limbwise).all()
    assert not (got == B.to_host(B.add_chain(da, db, 10), np.uint64)).all()


@pytest.mark.parametrize("m", [64, 256, 1024])
def test_mul_chain_matches_reference_six_multiplications(bigint, ref, m):
    """bi_mul_chain with p = 6 against convMul5Bench<U64bits, m, ipb, 6>."""
    import torch

    B = bigint
    n = 256
    da = B.to_device(uniform_limbs(930 + m, n, m))
    db = B.to_device(uniform_limbs(931 + m, n, m))
    rr = torch.empty_like(da)
    assert ref.lib().ref_mul6_u64(da.data_ptr(), db.data_ptr(), rr.data_ptr(), m, n, _sp()) == 0
    assert bool((B.mul_chain(da, db, 6) == rr).all())
