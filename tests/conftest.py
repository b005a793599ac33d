import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def cesa():
    """The product package with libcesa.so built for sm_103a."""
    from cuda_emicp_softassign_gb300 import build
    build.build()
    import cuda_emicp_softassign_gb300 as C
    C.lib()
    return C


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch


def soa_tensor(torch, P):
    from cuda_emicp_softassign_gb300 import cloud2data
    return torch.from_numpy(cloud2data(P)).cuda()


def rot_err_deg(A, B):
    from cuda_emicp_softassign_gb300.workloads import rotation_error_deg
    return rotation_error_deg(A, B)


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(np.abs(b).max(), floor, 1e-300)
    return float(np.abs(a - b).max() / den)
