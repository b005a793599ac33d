"""Bounded device-side waits: an expired wait ends the kernel with
CESA_ERR_TIMEOUT in its control block, and the context stays usable.

The probe runs the kernels' own grid barrier and mbarrier wait on barriers
that nothing completes (no fault, no trap: the waits give up after their
limit). A registration afterwards must still succeed."""
import numpy as np
import pytest

import cuda_emicp_softassign_gb300 as C


def test_self_test_rejects_bad_arguments(cesa):
    rc, _, _ = C.self_test_waits(2, 100)
    assert rc == C.CESA_ERR_INVALID_ARGUMENT
    rc, _, _ = C.self_test_waits(0, 0)
    assert rc == C.CESA_ERR_INVALID_ARGUMENT


@pytest.mark.gpu
@pytest.mark.parametrize("which,where", [(0, 90), (1, 91)])
def test_expired_wait_reports_timeout(torch_cuda, which, where):
    rc, status, wh = C.self_test_waits(which, 2000)
    assert rc == C.CESA_OK
    assert status == C.CESA_ERR_TIMEOUT
    assert wh == where


@pytest.mark.gpu
def test_registration_after_expired_waits(torch_cuda):
    for which in (0, 1):
        assert C.self_test_waits(which, 500)[0] == C.CESA_OK
    rng = np.random.default_rng(3)
    X = rng.random((300, 3)).astype(np.float32)
    a = np.deg2rad(10.0)
    Rt = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    Y = ((X - 0.01) @ Rt).astype(np.float32)  # X = Rt Y + 0.01
    R, t = C.emicp(X, Y, param=C.Params.default(sigma_inf=1e-4))
    assert np.degrees(np.arccos(np.clip((np.trace(R @ Rt.T) - 1) / 2, -1, 1))) < 0.5
