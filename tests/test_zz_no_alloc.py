"""The no-allocation EM-ICP entry point (cesa_emicp_device_noalloc).

It serves callers that cannot call cudaMalloc, such as a plugin without a
device heap of its own or a real-time pipeline that forbids allocation
after start-up. Its scratch is a fixed 16 MiB array inside libcesa.so.
This file is collected last, so that a run stopping at the first failure
has already run every other test. It also passes on its own in a fresh
process.
"""
import numpy as np
import pytest

from conftest import rot_err_deg, soa_tensor

pytestmark = pytest.mark.gpu


def _pose0(torch):
    return torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")


def test_noalloc_matches_device_entry_point_twice_in_a_row(cesa, torch_cuda):
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    _, X, Y, _, _ = W.make("c1_emicp_1007", seed=7)
    dX, dY = soa_tensor(torch, X), soa_tensor(torch, Y)
    ref = _pose0(torch)
    cesa.emicp_device(dX, dY, ref)
    torch.cuda.synchronize()
    assert cesa.stream_status() == cesa.CESA_OK
    R_ref = ref.cpu().numpy().astype(np.float64)
    extent = float(np.ptp(X, 0).max())
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        out = _pose0(torch)
        status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        rc = cesa.emicp_device_noalloc(dX, dY, out, d_status=status)
        assert rc == cesa.CESA_OK, cesa.status_string(rc)
        torch.cuda.synchronize()
        assert int(status.item()) == cesa.CESA_OK
        got = out.cpu().numpy().astype(np.float64)
        assert rot_err_deg(got[:9].reshape(3, 3), R_ref[:9].reshape(3, 3)) < 1e-3
        assert np.abs(got[9:] - R_ref[9:]).max() < 1e-5 * extent


def test_noalloc_rejects_problems_beyond_its_scratch(cesa, torch_cuda):
    torch = torch_cuda
    n = 400_000  # the EM-ICP workspace for 400k x 400k points exceeds 16 MiB
    dX = torch.zeros(3 * n, dtype=torch.float32, device="cuda")
    out = _pose0(torch)
    rc = cesa.emicp_device_noalloc(dX, dX, out)
    assert rc == cesa.CESA_ERR_NOALLOC_LIMIT
    assert "16 MiB" in cesa.status_string(rc)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), np.r_[np.eye(3).reshape(-1), np.zeros(3)].astype(np.float32))
