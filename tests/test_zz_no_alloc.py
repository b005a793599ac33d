"""The no-allocation EM-ICP entry point (cesa_emicp_device_noalloc).

It serves callers that cannot call cudaMalloc, such as a plugin without a
device heap of its own or a real-time pipeline that forbids allocation
after start-up. Its scratch is a fixed 16 MiB array inside libcesa.so.
This file is collected last, so that a run stopping at the first failure
has already run every other test. It also passes on its own in a fresh
process.

The kernels are deterministic and the no-allocation call runs the same
kernels with the same plan as cesa_emicp_device, so its pose must equal that
entry point's bit for bit; against the FP64 oracle it meets the usual
tolerances (R within 1e-3 degrees, t within 1e-5 x cloud extent).
"""
import numpy as np
import pytest

from conftest import rot_err_deg, soa_tensor

pytestmark = pytest.mark.gpu


def _pose0(torch):
    return torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")


def test_noalloc_matches_device_entry_point_twice_in_a_row(cesa, oracle, torch_cuda):
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    _, X, Y, _, _ = W.make("c1_emicp_1007", seed=7)
    dX, dY = soa_tensor(torch, X), soa_tensor(torch, Y)
    ref = _pose0(torch)
    cesa.emicp_device(dX, dY, ref)
    torch.cuda.synchronize()
    assert cesa.stream_status() == cesa.CESA_OK
    ref = ref.cpu().numpy()
    Ro, to, _ = oracle.emicp(X, Y)
    extent = float(np.ptp(X, 0).max())
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        out = _pose0(torch)
        status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
        rc = cesa.emicp_device_noalloc(dX, dY, out, d_status=status)
        assert rc == cesa.CESA_OK, cesa.status_string(rc)
        torch.cuda.synchronize()
        assert int(status.item()) == cesa.CESA_OK
        assert cesa.stream_status() == cesa.CESA_OK
        got = out.cpu().numpy()
        assert np.array_equal(got, ref)  # same kernels, same plan: bitwise
        got = got.astype(np.float64)
        assert rot_err_deg(got[:9].reshape(3, 3), Ro) < 1e-3
        assert np.abs(got[9:] - to).max() < 1e-5 * extent


def test_noalloc_status_on_a_user_stream_without_d_status(cesa, torch_cuda):
    """With d_status = NULL the status is read with cesa_stream_status(stream),
    which after a no-allocation call reads that call's status from the fixed
    scratch (not a stale workspace of an earlier call on the stream)."""
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    _, X, Y, _, _ = W.make("c1_emicp_1007", seed=8)
    dX, dY = soa_tensor(torch, X), soa_tensor(torch, Y)
    stream = torch.cuda.Stream()
    out, ref = _pose0(torch), _pose0(torch)
    torch.cuda.synchronize()  # inputs were written on the default stream
    rc = cesa.emicp_device_noalloc(dX, dY, out, stream=stream)
    assert rc == cesa.CESA_OK, cesa.status_string(rc)
    assert cesa.stream_status(stream) == cesa.CESA_OK
    cesa.emicp_device(dX, dY, ref, stream=stream)
    assert cesa.stream_status(stream) == cesa.CESA_OK
    out.copy_(_pose0(torch))
    torch.cuda.synchronize()
    rc = cesa.emicp_device_noalloc(dX, dY, out, stream=stream)
    assert rc == cesa.CESA_OK and cesa.stream_status(stream) == cesa.CESA_OK
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref.cpu().numpy())


def test_noalloc_accepts_100k_points(cesa, torch_cuda):
    """N = M = 100,000 fits the 16 MiB scratch on this GPU, and gives the
    device entry point's pose bitwise."""
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    X, Y, _, _ = W.uniform_pair(n=100_000, seed=9, max_deg=10.0, t_range=0.02)
    dX, dY = soa_tensor(torch, X), soa_tensor(torch, Y)
    p = cesa.Params.default(sigma_inf=1e-3)  # a shorter schedule (22 steps) keeps the test quick
    out = _pose0(torch)
    rc = cesa.emicp_device_noalloc(dX, dY, out, param=p)
    assert rc == cesa.CESA_OK, cesa.status_string(rc)
    ref = _pose0(torch)
    cesa.emicp_device(dX, dY, ref, param=p)
    torch.cuda.synchronize()
    assert cesa.stream_status() == cesa.CESA_OK
    assert np.array_equal(out.cpu().numpy(), ref.cpu().numpy())


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
