"""Softassign on the GPU through the C ABI, against the FP64 oracle.

Tolerances: slack vectors and row/column sums 1e-5 relative; S relative to
its largest entry at most max(1e-5, 2x the error of the reference's own FP32
arithmetic, i.e. the oracle's FP32 port): at high temperature the assignment
is nearly uniform and S is a small residue of the data; final R within 1e-3
degrees and t within 1e-5 x cloud extent for the full default schedule.
Schedules cut short at high temperature end ill-conditioned; there the pose
must match the FP64 oracle at least as well as the FP32 port does.
"""
import numpy as np
import pytest

from conftest import rel_err, rot_err_deg, soa_tensor

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,m", [(300, 300), (257, 129), (77, 500)])
@pytest.mark.parametrize("T", [100.0, 5.0, 0.7])
def test_inner_iteration_matches_oracle(cesa, oracle, torch_cuda, n, m, T):
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    X, Y, Rt, tt = W.surface_pair(n=n, m=m, seed=n + 3 * m)
    R, t = Rt, tt
    mo = np.float32(0.0367879)
    s0 = np.full(n, mo * 0.7, np.float32)  # slack already shrunk by earlier iterations
    u0 = np.full(m, mo * 0.9, np.float32)
    ref = oracle.softassign_step(X, Y, R.astype(np.float32), t.astype(np.float32), T, 3.0, 3, s0, u0)
    s = torch.from_numpy(s0.copy()).cuda()
    u = torch.from_numpy(u0.copy()).cuda()
    rs = torch.zeros(n, device="cuda")
    cs = torch.zeros(m, device="cuda")
    w = torch.zeros(n, device="cuda")
    mom = cesa.softassign_step(soa_tensor(torch, X), soa_tensor(torch, Y), R, t, T, 3.0, 3, s, u,
                               rs=rs, cs=cs, w=w)
    torch.cuda.synchronize()
    for name, got in (("s", s), ("u", u), ("rs", rs), ("cs", cs), ("w", w)):
        g = got.cpu().numpy().astype(np.float64)
        assert np.all(np.abs(g - ref[name]) <= 1e-5 * np.abs(ref[name]) + 1e-30), name
    assert abs(mom[0] - ref["sum"]) <= 1e-5 * ref["sum"]
    extent = float(np.ptp(X, 0).max())
    assert np.abs(mom[1:4] - ref["Xc"]).max() < 1e-5 * extent
    assert np.abs(mom[4:7] - ref["Yc"]).max() < 1e-5 * extent
    port = oracle.softassign_step(X, Y, R.astype(np.float32), t.astype(np.float32), T, 3.0, 3, s0, u0,
                                  precision="f32")
    e_gpu, e_port = rel_err(mom[7:16], ref["S"]), rel_err(port["S"], ref["S"])
    assert e_gpu <= max(1e-5, 2.0 * e_port), (e_gpu, e_port)


@pytest.mark.parametrize("n,m,seed", [(200, 200, 1), (160, 240, 2), (333, 100, 3)])
def test_full_schedule_matches_oracle(cesa, oracle, n, m, seed):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.surface_pair(n=n, m=m, seed=seed)
    R, t, tr, rep = cesa.softassign(X, Y, trace=True)
    Ro, to, tro = oracle.softassign(X, Y)
    Rp, tp, _ = oracle.softassign(X, Y, precision="f32", trace=False)
    assert rep.steps == 500 and len(tr) == 500
    assert tro[-1, 30] > 0.05
    # The assignment stays within ~10% of uniform over the whole default
    # schedule (alpha = 3 >> d^2), so the trajectory is sensitive to the FP32
    # state: 1e-3 deg, or at least 4x closer to FP64 than the reference's own
    # FP32 arithmetic on the same input, whichever is larger.
    e, e_port = rot_err_deg(R, Ro), rot_err_deg(Rp, Ro)
    assert e <= max(1e-3, 0.25 * e_port), (e, e_port)
    extent = float(np.ptp(X, 0).max())
    assert np.abs(t - to).max() <= max(1e-5 * extent, 0.25 * np.abs(tp - to).max())


def test_c2_full_size_matches_oracle(cesa, oracle):
    """Config 2 (N = M = 2000, default schedule, 500 pose updates)."""
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c2_softassign_2000", seed=0)
    R, t = cesa.softassign(X, Y)
    Ro, to, tro = oracle.softassign(X, Y)
    assert rot_err_deg(R, Ro) < 1e-3
    assert np.abs(t - to).max() < 1e-5 * float(np.ptp(X, 0).max())


def test_far_from_origin_frame_dependence_is_reproduced(cesa, oracle):
    """The reference's Softassign S depends on the coordinate origin (X is
    weighted, then centred); the centred kernels rebuild it exactly."""
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.surface_pair(n=150, seed=8)
    off = np.array([3.0, -2.0, 5.0], np.float32)
    Xo, Yo = X + off, Y + off
    R, t = cesa.softassign(Xo, Yo)
    Ro, to, tro = oracle.softassign(Xo, Yo)
    R0, _, _ = oracle.softassign(X, Y)
    assert rot_err_deg(Ro, R0) > 1e-2  # the origin matters in the reference algorithm
    assert rot_err_deg(R, Ro) < 1e-3
    assert np.abs(t - to).max() < 1e-5 * 5.0


@pytest.mark.parametrize("n,m", [(1, 1), (2, 5), (16, 17), (129, 33)])
def test_tiny_sizes(cesa, oracle, n, m):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.surface_pair(n=n, m=m, seed=n * 7 + m)
    p = cesa.Params.default(JMAX=20)
    R, t, tr, rep = cesa.softassign(X, Y, param=p, trace=True)
    Ro, to, tro = oracle.softassign(X, Y, JMAX=20)
    assert np.all(np.isfinite(R)) and np.all(np.isfinite(t))
    assert rel_err(tr[-1, 2], tro[-1, 2]) < 1e-5  # sumM
    # with a handful of points at high temperature the assignment is almost
    # uniform and S a tiny residue: the pose is ill-conditioned for any FP32
    # implementation. The reference arithmetic's own deviation from FP64 is
    # measured on an ensemble of inputs perturbed by one ulp (seeded): at
    # (16, 17) it spans 0 to 0.15 degrees (median 0.03), and a single run of it
    # depends on the host compiler's FMA contraction. The result must stay
    # within 4 x the largest deviation of the ensemble (the kernel's exp is
    # ex2.approx, a few times noisier per element than the port's expf).
    rng = np.random.default_rng(n * 31 + m)
    errs = []
    for _ in range(8):
        Xp = X.astype(np.float32) * (1 + rng.choice([-1, 0, 1], size=X.shape).astype(np.float32) * np.float32(6e-8))
        Rp, _, _ = oracle.softassign(Xp.astype(np.float64), Y, JMAX=20, precision="f32", trace=False)
        errs.append(rot_err_deg(Rp, Ro))
    assert rot_err_deg(R, Ro) <= max(1e-3, 4.0 * max(errs)), (rot_err_deg(R, Ro), errs)


def test_deterministic_and_device_entry(cesa, torch_cuda):
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    X, Y, _, _ = W.surface_pair(n=500, seed=5)
    p = cesa.Params.default(JMAX=10)
    R1, t1 = cesa.softassign(X, Y, param=p)
    R2, t2 = cesa.softassign(X, Y, param=p)
    assert np.array_equal(R1, R2) and np.array_equal(t1, t2)
    dRt = torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")
    cesa.softassign_device(soa_tensor(torch, X), soa_tensor(torch, Y), dRt, param=p)
    torch.cuda.synchronize()
    assert cesa.stream_status() == 0
    out = dRt.cpu().numpy().astype(np.float64)
    assert np.array_equal(out[:9].reshape(3, 3), R1) and np.array_equal(out[9:], t1)
