"""Dense FP64 restatements of EM-ICP and Softassign in torch, differentiable
by autograd -- TEST INFRASTRUCTURE ONLY.

Only tests/ may import this module. It is the FP64 dense reference gradient
of the adjoints: the whole N x M affinity matrix of every step is formed,
Horn's quaternion is the top eigenvector from torch.linalg.eigh, and autograd
differentiates the unrolled schedule. Runs on the CPU in float64.

The algorithm is that of emicp_cpu() (src/emicp_cpu.cpp:305-528, identical to
src/emicp.cu:443-669): per step, A_rc = exp(-|x_c - (R y_r + t)|^2 / sigma_p2),
C_r = sum_c A_rc + exp(-d_02 / sigma_p2), A <- sqrt(A / C_r) (or 1/N where
C_r <= 1e-6), lambda = A 1, X' = A X / lambda, weighted centres, S, and
findRTfromS (src/findRTfromS.cpp:33-159). sqrt(A / C) is written as
exp(-d^2 / (2 sigma_p2)) / sqrt(C), which is the same value and keeps the
derivative finite where A underflows.
"""
import numpy as np
import torch


def horn_matrix(S):
    """Horn's N from S[i + 3 j] (src/findRTfromS.cpp:38-74)."""
    Sxx, Sxy, Sxz, Syx, Syy, Syz, Szx, Szy, Szz = (S[k] for k in range(9))
    row0 = torch.stack([Sxx + Syy + Szz, Syz - Szy, Szx - Sxz, Sxy - Syx])
    row1 = torch.stack([Syz - Szy, Sxx - Syy - Szz, Sxy + Syx, Szx + Sxz])
    row2 = torch.stack([Szx - Sxz, Sxy + Syx, Syy - Sxx - Szz, Syz + Szy])
    row3 = torch.stack([Sxy - Syx, Szx + Sxz, Syz + Szy, Szz - Sxx - Syy])
    return torch.stack([row0, row1, row2, row3])


def quat_to_R(q):
    q0, qx, qy, qz = q[0], q[1], q[2], q[3]
    return torch.stack([
        torch.stack([q0 * q0 + qx * qx - qy * qy - qz * qz, 2 * (qx * qy - q0 * qz), 2 * (qx * qz + q0 * qy)]),
        torch.stack([2 * (qy * qx + q0 * qz), q0 * q0 - qx * qx + qy * qy - qz * qz, 2 * (qy * qz - q0 * qx)]),
        torch.stack([2 * (qz * qx - q0 * qy), 2 * (qz * qy + q0 * qx), q0 * q0 - qx * qx - qy * qy + qz * qz]),
    ])


def sigma_schedule(sigma_p2=0.01, sigma_inf=1e-5, sigma_factor=0.9):
    """The sigma_p2 values of the steps, stepped in FP32 (src/emicp.cu:443,668)."""
    out = []
    s = np.float32(sigma_p2)
    while s > np.float32(sigma_inf):
        out.append(float(s))
        s = np.float32(s * np.float32(sigma_factor))
    return out


def emicp(X, Y, R0, t0, sigma_p2=0.01, sigma_inf=1e-5, sigma_factor=0.9, d_02=0.01):
    """X (N,3), Y (M,3), R0 (3,3), t0 (3) float64 tensors -> (R, t)."""
    N = X.shape[0]
    R, t = R0, t0
    for s2 in sigma_schedule(sigma_p2, sigma_inf, sigma_factor):
        Z = Y @ R.T + t
        d2 = ((Z[:, None, :] - X[None, :, :]) ** 2).sum(-1)  # (M, N)
        e = torch.exp(-d2 / (2.0 * s2))
        C = (e * e).sum(1) + np.exp(-d_02 / s2)
        branch = ~(C > 1e-6)
        Cs = torch.where(branch, torch.ones_like(C), C)
        A = torch.where(branch[:, None], torch.full_like(e, 1.0 / N), e / torch.sqrt(Cs)[:, None])
        lam = A.sum(1)
        U = A @ X  # lambda X'
        L = lam.sum()
        Xc = U.sum(0) / L
        Yc = (lam[:, None] * Y).sum(0) / L
        Sm = (U - lam[:, None] * Xc).T @ (Y - Yc)  # S_ij = sum (u_i - lambda Xc_i)(y_j - Yc_j)
        S = Sm.T.reshape(-1)  # S[i + 3 j]
        w, V = torch.linalg.eigh(horn_matrix(S))
        q = V[:, -1]
        R = quat_to_R(q)
        t = Xc - R @ Yc
    return R, t


def so3_exp(w):
    th = torch.linalg.norm(w)
    K = torch.zeros(3, 3, dtype=w.dtype)
    K = torch.stack([torch.stack([K[0, 0], -w[2], w[1]]), torch.stack([w[2], K[1, 1], -w[0]]),
                     torch.stack([-w[1], w[0], K[2, 2]])])
    if float(th.detach()) < 1e-12:
        return torch.eye(3, dtype=w.dtype) + K
    return torch.eye(3, dtype=w.dtype) + torch.sin(th) / th * K + (1 - torch.cos(th)) / th ** 2 * (K @ K)


def pose_loss_grads(X, Y, R0, t0, R_true, t_true, **sched):
    """Loss |R - R_true|_F^2 + |t - t_true|^2 of the registration from the
    initial pose exp(w) R0, t0 + v at w = v = 0, and its gradients with
    respect to X, Y, w and v (numpy float64)."""
    Xt = torch.tensor(np.asarray(X, np.float64), requires_grad=True)
    Yt = torch.tensor(np.asarray(Y, np.float64), requires_grad=True)
    w = torch.zeros(3, dtype=torch.float64, requires_grad=True)
    v = torch.zeros(3, dtype=torch.float64, requires_grad=True)
    R0t = torch.tensor(np.asarray(R0, np.float64))
    t0t = torch.tensor(np.asarray(t0, np.float64))
    R, t = emicp(Xt, Yt, so3_exp(w) @ R0t, t0t + v, **sched)
    loss = ((R - torch.tensor(R_true)) ** 2).sum() + ((t - torch.tensor(t_true)) ** 2).sum()
    loss.backward()
    return (float(loss.detach()), Xt.grad.numpy(), Yt.grad.numpy(), w.grad.numpy(), v.grad.numpy(),
            R.detach().numpy(), t.detach().numpy())


def loss_value(X, Y, R0, t0, R_true, t_true, **sched):
    with torch.no_grad():
        R, t = emicp(torch.tensor(X, dtype=torch.float64), torch.tensor(Y, dtype=torch.float64),
                     torch.tensor(R0, dtype=torch.float64), torch.tensor(t0, dtype=torch.float64), **sched)
        return float(((R - torch.tensor(R_true)) ** 2).sum() + ((t - torch.tensor(t_true)) ** 2).sum())


def softassign_moutlier(T_0):
    """The slack's initial value 1/sqrt(T_0) e^-1 in FP32 (src/softassign.cu:385-390)."""
    return float(np.float32(1.0 / np.sqrt(np.float32(T_0)) * np.exp(np.float32(-1.0))))


def _softassign_updates(X, Y, R, t, s, u, Tv, I0, I1, alpha):
    for _ in range(I0):
        Z = Y @ R.T + t
        d2 = ((X[:, None, :] - Z[None, :, :]) ** 2).sum(-1)  # (N, M)
        Mx = torch.exp(-(d2 - float(np.float32(alpha))) / Tv) / np.sqrt(Tv)
        for _ in range(I1):
            rs = Mx.sum(1) + s
            Mx = Mx / rs[:, None]
            s = s / rs
            cs = Mx.sum(0) + u
            Mx = Mx / cs[None, :]
            u = u / cs
        w = Mx.sum(1)
        sumM = w.sum()
        Xc = (w[:, None] * X).sum(0) / sumM
        Yc = (cs[:, None] * Y).sum(0) / sumM
        Xw = w[:, None] * X - Xc
        Yw = cs[:, None] * Y - Yc
        Sm = Xw.T @ (Mx @ Yw)  # S_ij = sum_r xw_ri (M Yw)_rj
        S = Sm.T.reshape(-1)  # S[i + 3 j]
        _, V = torch.linalg.eigh(horn_matrix(S))
        q = V[:, -1]
        R = quat_to_R(q)
        t = Xc - R @ Yc
    return R, t, s, u


def softassign(X, Y, R0, t0, JMAX=100, I0=5, I1=3, alpha=3.0, T_0=100.0, TFACTOR=0.95, moutlier=None,
               checkpoint=False):
    """Annealed Softassign, as oracle_softassign (src/softassign.cu:486-822):
    per update M = exp(-(|x_r - (R y_c + t)|^2 - alpha)/T)/sqrt(T), I1 slack
    row/column normalisations with s and u carried across all updates, w = M 1,
    Xc = sum w x / sum w, Yc = sum cs y / sum w (cs: the last column sums
    before their normalisation), S = (w x - Xc)^T M (cs y - Yc) and Horn's
    pose. X (N,3), Y (M,3), R0, t0 float64 tensors -> (R, t). checkpoint:
    keep only (R, t, s, u) per T step for autograd and recompute the T step's
    updates in the backward (bounded memory for long schedules)."""
    N, M = X.shape[0], Y.shape[0]
    if moutlier is None:
        moutlier = softassign_moutlier(T_0)
    s = torch.full((N,), moutlier, dtype=X.dtype)
    u = torch.full((M,), moutlier, dtype=X.dtype)
    R, t = R0, t0
    T = np.float32(T_0)
    for _ in range(JMAX):
        if checkpoint:
            from torch.utils.checkpoint import checkpoint as ckpt
            R, t, s, u = ckpt(_softassign_updates, X, Y, R, t, s, u, float(T), I0, I1, alpha, use_reentrant=False)
        else:
            R, t, s, u = _softassign_updates(X, Y, R, t, s, u, float(T), I0, I1, alpha)
        T = np.float32(T * np.float32(TFACTOR))
    return R, t


def softassign_loss_grads(X, Y, R0, t0, R_true, t_true, **sched):
    """As pose_loss_grads, for Softassign."""
    Xt = torch.tensor(np.asarray(X, np.float64), requires_grad=True)
    Yt = torch.tensor(np.asarray(Y, np.float64), requires_grad=True)
    w = torch.zeros(3, dtype=torch.float64, requires_grad=True)
    v = torch.zeros(3, dtype=torch.float64, requires_grad=True)
    R0t = torch.tensor(np.asarray(R0, np.float64))
    t0t = torch.tensor(np.asarray(t0, np.float64))
    R, t = softassign(Xt, Yt, so3_exp(w) @ R0t, t0t + v, **sched)
    loss = ((R - torch.tensor(R_true)) ** 2).sum() + ((t - torch.tensor(t_true)) ** 2).sum()
    loss.backward()
    return (float(loss.detach()), Xt.grad.numpy(), Yt.grad.numpy(), w.grad.numpy(), v.grad.numpy(),
            R.detach().numpy(), t.detach().numpy())
