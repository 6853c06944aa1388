"""Shared test setup: import paths, the `gpu` marker and common fixtures."""
import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "big-int_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(REPO, "tests", "golden", "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def bigint():
    """The CUDA library, built in-tree; GPU tests fail (not skip) if it is absent."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import bigint_gb300 as B

    B.build()
    B.lib()
    return B


def limbs(rows, bits):
    return np.array(rows, dtype=np.uint64 if bits == 64 else np.uint32)
