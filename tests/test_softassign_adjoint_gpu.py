"""Adjoint of Softassign (cesa_softassign_forward_device /
cesa_softassign_backward_device) against the FP64 dense reference gradient
(oracle/torch_ref.py: the unrolled annealing loop with N x M matrices, slack
carried across updates and torch.linalg.eigh, differentiated by autograd).
The reference is pinned here: its forward equals the FP64 oracle's and its
gradient equals FP64 central differences of its own forward (h = 1e-6; the
oracle's Horn solve stops at a tolerance, so differences of the oracle are
noisy below h = 1e-5).

Surface views (the Softassign workload's generator) at N = M = 200 and a
shortened schedule (JMAX = 20, I0 = 5, I1 = 3, T from 100 down by 0.8 per
step: 100 pose updates). Loss = |R - R_true|_F^2 + |t - t_true|^2.
Tolerance: each gradient block (dL/dX, dL/dY, dL/d se(3)) within 5e-3 of the
reference relative to the block's largest entry; the forward runs in FP32
and the backward accumulates 100 updates of FP32 round-off. The backward's
two executions (softassign_backward_form: one persistent launch, the default
at these sizes, and each update's launch sequence, the default for large
clouds, whose gradient sweep owns the rows and sums the columns by a
transpose) are both checked.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHED = dict(JMAX=20, I0=5, I1=3, T_0=100.0, TFACTOR=0.8)
TOL = 5e-3


def _pair(n, m, seed):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, Rt, tt = W.surface_pair(n=n, m=m, seed=seed)
    return X.astype(np.float32).astype(np.float64), Y.astype(np.float32).astype(np.float64), Rt, tt


@pytest.fixture(scope="module")
def case():
    return _pair(200, 200, 1)


@pytest.fixture(scope="module")
def reference(case):
    from oracle import torch_ref as T
    X, Y, Rt, tt = case
    return T.softassign_loss_grads(X, Y, np.eye(3), np.zeros(3), Rt, tt, **SCHED)


def _loss_t(X, Y, R0, t0, Rt, tt, **sched):
    import torch
    from oracle import torch_ref as T
    with torch.no_grad():
        R, t = T.softassign(torch.tensor(X), torch.tensor(Y), torch.tensor(R0), torch.tensor(t0), **sched)
    return float(((R - torch.tensor(Rt)) ** 2).sum() + ((t - torch.tensor(tt)) ** 2).sum())


def _rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


def _se3(w, v):
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    Rw = np.eye(3) + (np.sin(th) / th * K + (1 - np.cos(th)) / th ** 2 * K @ K if th > 0 else K)
    return Rw, np.asarray(v, np.float64)


def test_reference_pinned(case, reference, oracle):
    X, Y, Rt, tt = case
    loss, gX, gY, gw, gv, R, t = reference
    Ro, to, _ = oracle.softassign(X, Y, trace=False, **SCHED)
    assert np.abs(R - Ro).max() < 1e-10 and np.abs(t - to).max() < 1e-10
    rng = np.random.default_rng(1)
    h = 1e-6
    for name, P, G in (("X", X, gX), ("Y", Y, gY)):
        for _ in range(3):
            i, k = int(rng.integers(len(P))), int(rng.integers(3))
            Pp, Pm = P.copy(), P.copy()
            Pp[i, k] += h
            Pm[i, k] -= h
            a = (Pp, Y) if name == "X" else (X, Pp)
            b = (Pm, Y) if name == "X" else (X, Pm)
            fd = (_loss_t(*a, np.eye(3), np.zeros(3), Rt, tt, **SCHED) -
                  _loss_t(*b, np.eye(3), np.zeros(3), Rt, tt, **SCHED)) / (2 * h)
            assert abs(fd - G[i, k]) <= 1e-6 * np.abs(G).max(), (name, i, k, fd, G[i, k])
    for k in range(6):
        d = np.zeros(6)
        d[k] = 1e-4
        vals = [_loss_t(X, Y, *_se3(sgn * d[:3], sgn * d[3:]), Rt, tt, **SCHED) for sgn in (1, -1)]
        fd = (vals[0] - vals[1]) / 2e-4
        ad = gw[k] if k < 3 else gv[k - 3]
        assert abs(fd - ad) <= 1e-3 * max(np.abs(gw).max(), np.abs(gv).max(), 1e-12), (k, fd, ad)


FORMS = ("persistent", "launches")


def _gpu_grads(cesa, torch, X, Y, R0, t0, Rt, tt, form="persistent", **sched):
    from cuda_emicp_softassign_gb300.autograd import se3_gradient, softassign_autograd
    Xd = torch.tensor(X, dtype=torch.float32, device="cuda", requires_grad=True)
    Yd = torch.tensor(Y, dtype=torch.float32, device="cuda", requires_grad=True)
    R0d = torch.tensor(R0, dtype=torch.float32, device="cuda", requires_grad=True)
    t0d = torch.tensor(t0, dtype=torch.float32, device="cuda", requires_grad=True)
    code = {"persistent": cesa.SA_BACKWARD_PERSISTENT, "launches": cesa.SA_BACKWARD_LAUNCHES}[form]
    R, t = softassign_autograd(Xd, Yd, R0d, t0d, cesa.Params.default(softassign_backward_form=code, **sched))
    loss = ((R - torch.tensor(Rt, dtype=torch.float32, device="cuda")) ** 2).sum() + \
        ((t - torch.tensor(tt, dtype=torch.float32, device="cuda")) ** 2).sum()
    loss.backward()
    gw, gv = se3_gradient(R0d.detach(), R0d.grad, t0d.grad)
    return (R.detach().cpu().numpy(), t.detach().cpu().numpy(), Xd.grad.cpu().numpy(), Yd.grad.cpu().numpy(),
            np.r_[gw.cpu().numpy(), gv.cpu().numpy()])


def test_forward_equals_the_matrix_free_entry_point(cesa, torch_cuda, case):
    X, Y, Rt, tt = case
    R, t, _, _, _ = _gpu_grads(cesa, torch_cuda, X, Y, np.eye(3), np.zeros(3), Rt, tt, **SCHED)
    p = cesa.Params.default(sinkhorn_form=cesa.SINKHORN_MATRIX_FREE, **SCHED)
    Rp, tp = cesa.softassign(X.astype(np.float32), Y.astype(np.float32), param=p)
    assert np.array_equal(R.astype(np.float64), Rp) and np.array_equal(t.astype(np.float64), tp)


@pytest.mark.parametrize("form", FORMS)
def test_gpu_adjoint_matches_fp64_reference(cesa, torch_cuda, case, reference, form):
    X, Y, Rt, tt = case
    _, gX, gY, gw, gv, _, _ = reference
    _, _, gXd, gYd, g6 = _gpu_grads(cesa, torch_cuda, X, Y, np.eye(3), np.zeros(3), Rt, tt, form=form, **SCHED)
    assert _rel(gXd, gX) < TOL, _rel(gXd, gX)
    assert _rel(gYd, gY) < TOL, _rel(gYd, gY)
    assert _rel(g6, np.r_[gw, gv]) < TOL, (g6, np.r_[gw, gv])


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n,m,I1,seed", [(333, 157, 1, 2), (120, 517, 5, 3), (37, 1000, 3, 4)])
def test_ragged_sizes_and_inner_counts(cesa, torch_cuda, n, m, I1, seed, form):
    """One annealing step of I0 = 2 updates from a perturbed pose: ragged tiles,
    I1 = 1 (one column pass) and I1 = 5 (14 rank-1 terms: two gradient groups)."""
    from oracle import torch_ref as T
    X, Y, Rt, tt = _pair(n, m, seed)
    sched = dict(JMAX=1, I0=2, I1=I1, T_0=0.05, TFACTOR=0.9)
    R0, t0 = _se3(np.array([0.05, -0.02, 0.03]), np.array([0.01, 0.0, -0.01]))
    _, gX, gY, gw, gv, _, _ = T.softassign_loss_grads(X, Y, R0, t0, Rt, tt, **sched)
    _, _, gXd, gYd, g6 = _gpu_grads(cesa, torch_cuda, X, Y, R0, t0, Rt, tt, form=form, **sched)
    assert np.all(np.isfinite(gXd)) and np.all(np.isfinite(gYd)) and np.all(np.isfinite(g6))
    assert _rel(gXd, gX) < TOL, _rel(gXd, gX)
    assert _rel(gYd, gY) < TOL, _rel(gYd, gY)
    assert _rel(g6, np.r_[gw, gv]) < TOL, (g6, np.r_[gw, gv])


def test_c5_copy_full_schedule(cesa, torch_cuda):
    """The Softassign adjoint workload's check: its generator at N = M = 300 and
    the default schedule (JMAX = 100, I0 = 5, I1 = 3: 500 updates from T = 100).
    The reference (checkpointed per T step) is pinned by central differences of
    its forward at two X and two Y coordinates. Annealing from T = 100 erases
    the initial pose (|dL/d se(3)| ~ 1e-8), so that block is checked in
    absolute terms, within 5e-3 of the largest |dL/dY|."""
    from cuda_emicp_softassign_gb300 import workloads as W
    from oracle import torch_ref as T
    _, X, Y, Rt, tt = W.make("c5_softassign_20000", seed=0, n=300)
    X = X.astype(np.float32).astype(np.float64)
    Y = Y.astype(np.float32).astype(np.float64)
    _, gX, gY, gw, gv, _, _ = T.softassign_loss_grads(X, Y, np.eye(3), np.zeros(3), Rt, tt, checkpoint=True)
    rng = np.random.default_rng(5)
    h = 1e-6
    for name, P, G in (("X", X, gX), ("Y", Y, gY)):
        for _ in range(2):
            i, k = int(rng.integers(len(P))), int(rng.integers(3))
            Pp, Pm = P.copy(), P.copy()
            Pp[i, k] += h
            Pm[i, k] -= h
            a = (Pp, Y) if name == "X" else (X, Pp)
            b = (Pm, Y) if name == "X" else (X, Pm)
            fd = (_loss_t(*a, np.eye(3), np.zeros(3), Rt, tt) - _loss_t(*b, np.eye(3), np.zeros(3), Rt, tt)) / (2 * h)
            assert abs(fd - G[i, k]) <= 1e-6 * np.abs(G).max(), (name, i, k, fd, G[i, k])
    _, _, gXd, gYd, g6 = _gpu_grads(cesa, torch_cuda, X, Y, np.eye(3), np.zeros(3), Rt, tt)
    assert _rel(gXd, gX) < TOL, _rel(gXd, gX)
    assert _rel(gYd, gY) < TOL, _rel(gYd, gY)
    assert np.abs(g6 - np.r_[gw, gv]).max() <= TOL * np.abs(gY).max(), (g6, np.r_[gw, gv])
