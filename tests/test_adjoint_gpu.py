"""Adjoint of EM-ICP (cesa_emicp_forward_device / cesa_emicp_backward_device)
against the FP64 dense reference gradient (oracle/torch_ref.py: the unrolled
schedule with N x M affinities and torch.linalg.eigh, differentiated by
autograd), which is itself checked here against FP64 central differences
(h = 1e-6) and against the FP64 oracle's forward pose.

Config 3's check runs on an N = M = 500 copy (surface views, 5% outliers,
rotation up to 20 degrees). Loss = |R - R_true|_F^2 + |t - t_true|^2.
Tolerance: each gradient block (dL/dX, dL/dY, dL/d se(3)) within 2e-3 of the
reference relative to the block's largest entry; the forward pass runs in
FP32 and the gradient accumulates 66 steps of FP32 round-off. Every work
decomposition of the backward (emicp_backward_layout: by size, units of
slices, ranged task runs; at this size AUTO takes the slices, and the ranged
layout leaves most blocks without a task) is checked.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c3_small():
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, Rt, tt = W.make("c3_emicp_40097", seed=0, n=500)
    X = X.astype(np.float32).astype(np.float64)
    Y = Y.astype(np.float32).astype(np.float64)
    return X, Y, Rt, tt


@pytest.fixture(scope="module")
def reference(c3_small):
    from oracle import torch_ref as T
    X, Y, Rt, tt = c3_small
    return T.pose_loss_grads(X, Y, np.eye(3), np.zeros(3), Rt, tt)


def test_reference_gradient_pinned(c3_small, reference, oracle):
    from oracle import torch_ref as T
    X, Y, Rt, tt = c3_small
    loss, gX, gY, gw, gv, R, t = reference
    Ro, to, _ = oracle.emicp(X, Y)
    assert np.abs(R - Ro).max() < 1e-10 and np.abs(t - to).max() < 1e-10
    rng = np.random.default_rng(1)
    h = 1e-6
    for name, P, G in (("X", X, gX), ("Y", Y, gY)):
        for _ in range(4):
            i, k = int(rng.integers(len(P))), int(rng.integers(3))
            Pp, Pm = P.copy(), P.copy()
            Pp[i, k] += h
            Pm[i, k] -= h
            a = (Pp, Y) if name == "X" else (X, Pp)
            b = (Pm, Y) if name == "X" else (X, Pm)
            fd = (T.loss_value(*a, np.eye(3), np.zeros(3), Rt, tt) - T.loss_value(*b, np.eye(3), np.zeros(3), Rt, tt)) / (2 * h)
            assert abs(fd - G[i, k]) <= 1e-6 * np.abs(G).max() + 1e-9, (name, i, k, fd, G[i, k])
    # se(3) of the initial pose, central differences of the FP64 oracle
    for k in range(6):
        d = np.zeros(6)
        d[k] = h
        vals = []
        for sgn in (1, -1):
            w = sgn * d[:3]
            th = np.linalg.norm(w)
            K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
            Rw = np.eye(3) + (np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K if th > 0 else K)
            Ro, to, _ = oracle.emicp(X, Y, R0=Rw, t0=sgn * d[3:], trace=False)
            vals.append(((Ro - Rt) ** 2).sum() + ((to - tt) ** 2).sum())
        fd = (vals[0] - vals[1]) / (2 * h)
        ad = gw[k] if k < 3 else gv[k - 3]
        assert abs(fd - ad) <= 1e-5 * max(np.abs(gw).max(), np.abs(gv).max()), (k, fd, ad)


@pytest.mark.parametrize("layout", ["auto", "slices", "ranged"])
def test_gpu_adjoint_matches_fp64_reference(cesa, torch_cuda, c3_small, reference, layout):
    from cuda_emicp_softassign_gb300.autograd import emicp_autograd, se3_gradient
    torch = torch_cuda
    p = cesa.Params.default(emicp_backward_layout={"auto": cesa.LAYOUT_AUTO, "slices": cesa.LAYOUT_SLICES,
                                                   "ranged": cesa.LAYOUT_RANGED}[layout])
    X, Y, Rt, tt = c3_small
    loss_ref, gX, gY, gw, gv, Rr, tr = reference
    Xd = torch.tensor(X, dtype=torch.float32, device="cuda", requires_grad=True)
    Yd = torch.tensor(Y, dtype=torch.float32, device="cuda", requires_grad=True)
    R0 = torch.eye(3, device="cuda", requires_grad=True)
    t0 = torch.zeros(3, device="cuda", requires_grad=True)
    R, t = emicp_autograd(Xd, Yd, R0, t0, p)
    # the forward equals the plain device entry point
    Rp, tp = cesa.emicp(X.astype(np.float32), Y.astype(np.float32))
    assert np.array_equal(R.detach().cpu().numpy().astype(np.float64), Rp)
    loss = ((R - torch.tensor(Rt, dtype=torch.float32, device="cuda")) ** 2).sum() + \
        ((t - torch.tensor(tt, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    gw_d, gv_d = se3_gradient(R0.detach(), R0.grad, t0.grad)

    def rel(a, b):
        return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))

    assert rel(Xd.grad.cpu().numpy(), gX) < 2e-3
    assert rel(Yd.grad.cpu().numpy(), gY) < 2e-3
    g6 = np.r_[gw, gv]
    assert rel(np.r_[gw_d.cpu().numpy(), gv_d.cpu().numpy()], g6) < 2e-3


def test_sm_pairs_leave_gradients_unchanged(cesa, torch_cuda, monkeypatch):
    """At config 3's size the backward's slice units are dealt unequally to
    the two blocks of each SM (the larger part to the block the SM favours);
    that decides only which block computes a unit, so the gradients are
    bitwise those of the even deal (CESA_SM_PAIRS=0 set between the forward
    and the backward, so that both backwards differentiate the same taped
    forward)."""
    from cuda_emicp_softassign_gb300 import workloads as W
    from cuda_emicp_softassign_gb300.autograd import emicp_autograd
    torch = torch_cuda
    _, X, Y, _, _ = W.make("c3_emicp_40097", seed=0)
    p = cesa.Params.default(emicp_backward_layout=cesa.LAYOUT_SLICES)

    def grads(even_backward):
        Xd = torch.tensor(X, dtype=torch.float32, device="cuda", requires_grad=True)
        Yd = torch.tensor(Y, dtype=torch.float32, device="cuda", requires_grad=True)
        R0 = torch.eye(3, device="cuda", requires_grad=True)
        t0 = torch.zeros(3, device="cuda", requires_grad=True)
        R, t = emicp_autograd(Xd, Yd, R0, t0, p)
        loss = (R ** 2).sum() + (t ** 2).sum()
        if even_backward:
            monkeypatch.setenv("CESA_SM_PAIRS", "0")
        loss.backward()
        monkeypatch.delenv("CESA_SM_PAIRS", raising=False)
        return [v.detach().cpu().numpy() for v in (Xd.grad, Yd.grad, R0.grad, t0.grad)]

    paired = grads(False)
    again = grads(False)
    even = grads(True)
    for a, b, c in zip(paired, again, even):
        assert np.isfinite(a).all()
        assert np.array_equal(a, b) and np.array_equal(a, c)
