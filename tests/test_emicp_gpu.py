"""EM-ICP on the GPU through the C ABI, against the FP64 oracle.

Tolerances (FP32 kernels vs the FP64 restatement of the same algorithm):
  * per-row C_r, lambda_r, lambda_r X'_r: worst relative error at most
    max(1e-5, 2x the worst error of the reference's own FP32 arithmetic (the
    oracle's FP32 port) on the same inputs). At small sigma the FP32 rounding
    of R*y + t alone moves exp(-d^2/sigma^2) by up to ~6e-5 per row, in the
    reference as here;
  * moments (sum lambda, Xc, Yc, S): 1e-5 relative to their magnitude;
  * final R within 1e-3 degrees, t within 1e-5 x cloud extent.
"""
import os

import numpy as np
import pytest

from conftest import rel_err, rot_err_deg, soa_tensor

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _pose(seed, deg=5.0):
    from cuda_emicp_softassign_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    return W.random_rotation(rng, deg), rng.uniform(-0.02, 0.02, 3)


# 64 x 80000: a block's share of the rows exceeds one pass of 256 threads
@pytest.mark.parametrize("n,m", [(1007, 1007), (300, 200), (129, 777), (64, 80000)])
@pytest.mark.parametrize("sigma_p2", [1e-2, 1e-3, 1e-4, 1.06e-5])
def test_estep_rows_and_moments(cesa, oracle, torch_cuda, n, m, sigma_p2):
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    X, Y, Rt, tt = W.uniform_pair(n=n, m=m, seed=n + m)
    R, t = Rt, tt  # pose near the solution: many significant elements per row
    if sigma_p2 >= 1e-3:
        R, t = _pose(7)
    dX, dY = soa_tensor(torch, X), soa_tensor(torch, Y)
    rows = torch.zeros(m * 5, dtype=torch.float32, device="cuda")
    mom = cesa.emicp_step(dX, dY, R, t, sigma_p2, 0.01, row_out=rows)
    torch.cuda.synchronize()
    got = rows.cpu().numpy().reshape(m, 5)
    ref = oracle.emicp_step(X, Y, R.astype(np.float32), t.astype(np.float32), sigma_p2, 0.01)
    port = oracle.emicp_step(X, Y, R.astype(np.float32), t.astype(np.float32), sigma_p2, 0.01,
                             precision="f32")

    def worst(a, b, floor):
        return float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max())

    for col, key, floor in ((0, "C", 1e-30), (1, "lam", 1e-3)):
        e_gpu = worst(got[:, col], ref[key], floor)
        e_port = worst(port[key], ref[key], floor)
        assert e_gpu <= max(1e-5, 2.0 * e_port), (key, e_gpu, e_port)
    e_gpu = rel_err(got[:, 2:5], ref["U"])
    e_port = rel_err(port["U"], ref["U"])
    assert e_gpu <= max(1e-5, 2.0 * e_port), ("U", e_gpu, e_port)
    assert abs(mom[0] - ref["sum"]) <= 1e-5 * ref["sum"]
    extent = float(np.ptp(X, 0).max())
    assert np.abs(mom[1:4] - ref["Xc"]).max() < 1e-5 * extent
    assert np.abs(mom[4:7] - ref["Yc"]).max() < 1e-5 * extent
    assert rel_err(mom[7:16], ref["S"]) < 1e-5


def test_c1_full_registration_matches_oracle(cesa, oracle):
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, Rt, tt = W.make("c1_emicp_1007", seed=0)
    R, t, tr, rep = cesa.emicp(X, Y, trace=True)
    Ro, to, tro = oracle.emicp(X, Y)
    assert rep.steps == 66 and len(tr) == 66
    extent = float(np.ptp(X, 0).max())
    assert rot_err_deg(R, Ro) < 1e-3
    assert np.abs(t - to).max() < 1e-5 * extent
    # per-step agreement of the trajectory
    for k in range(66):
        assert rot_err_deg(tr[k, 18:27].reshape(3, 3), tro[k, 18:27].reshape(3, 3)) < 1e-3, k
        assert rel_err(tr[k, 9:18], tro[k, 9:18]) < 1e-4, k
    assert rot_err_deg(R, Rt) < 0.1  # converged (EM-ICP's own bias is ~0.01 deg here)


def test_reference_golden_cases(cesa):
    g = np.load(os.path.join(GOLD, "emicp_reference.npz"))
    for name in g["names"]:
        X, Y = g["emicp_%s_X" % name], g["emicp_%s_Y" % name]
        R, t = cesa.emicp(X, Y)
        extent = float(np.ptp(X, 0).max())
        assert rot_err_deg(R, g["emicp_%s_R" % name]) < 1e-3, name
        assert np.abs(t - g["emicp_%s_t" % name]).max() < 2e-5 * extent, name


@pytest.mark.parametrize("n,m", [(1, 1), (2, 3), (15, 16), (16, 17), (33, 127), (128, 128), (129, 1),
                                 (513, 200), (1000, 2049), (64, 80000)])
def test_ragged_sizes_match_oracle(cesa, oracle, n, m):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.uniform_pair(n=n, m=m, seed=3 * n + m, max_deg=10.0, t_range=0.03)
    p = cesa.Params.default(sigma_inf=2e-4)  # 38 steps
    R, t, tr, rep = cesa.emicp(X, Y, param=p, trace=True)
    Ro, to, tro = oracle.emicp(X, Y, sigma_inf=2e-4)
    assert rep.steps == len(tro)
    assert np.all(np.isfinite(R)) and np.all(np.isfinite(t))
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-5)
    extent = max(float(np.ptp(X, 0).max()), 1e-3)
    # weighted centres agree at every step; with a single point S is zero and
    # R is undefined (the oracle and the kernel follow different round-off),
    # but every pose still maps Yc onto Xc
    assert np.abs(tr[:, 3:9] - tro[:, 3:9]).max() < 1e-5 * extent + 1e-6
    Rl = tr[-1, 18:27].reshape(3, 3)
    assert np.abs(Rl @ tr[-1, 6:9] + tr[-1, 27:30] - tr[-1, 3:6]).max() < 1e-5
    if tro[:, 30].min() > 1e-3 and min(n, m) > 1:
        assert rot_err_deg(R, Ro) < 1e-3, (n, m)
        assert np.abs(t - to).max() < 1e-5 * extent, (n, m)


def test_far_from_origin_coordinates(cesa, oracle):
    """Scanner-frame offsets: centring keeps the FP32 kernels accurate."""
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.uniform_pair(n=500, seed=21, max_deg=10.0, t_range=0.03)
    off = np.array([1200.0, -350.0, 80.0], np.float32)
    Xo, Yo = X + off, Y + off
    R, t = cesa.emicp(Xo, Yo)
    Ro, to, _ = oracle.emicp(Xo.astype(np.float32), Yo.astype(np.float32))
    assert rot_err_deg(R, Ro) < 1e-3
    # t absorbs (I - R) off; compare at the data's own scale
    assert np.abs(t - to).max() < 1e-5 * 1200.0


def test_degenerate_rows_take_reference_branch(cesa, oracle, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(3)
    X = rng.uniform(0, 1, (40, 3)).astype(np.float32)
    Y = (rng.uniform(0, 1, (30, 3)) + 50.0).astype(np.float32)
    rows = torch.zeros(30 * 5, dtype=torch.float32, device="cuda")
    cesa.emicp_step(soa_tensor(torch, X), soa_tensor(torch, Y), np.eye(3), np.zeros(3), 1e-4, 0.01,
                    row_out=rows)
    got = rows.cpu().numpy().reshape(30, 5)
    assert np.all(got[:, 0] <= 1e-6)
    assert np.allclose(got[:, 1], 1.0)
    assert np.allclose(got[:, 2:5], X.astype(np.float64).mean(0), atol=1e-5)


def test_host_and_device_entry_points_agree_bitwise(cesa, torch_cuda):
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    _, X, Y, _, _ = W.make("c1_emicp_1007", seed=4)
    R1, t1 = cesa.emicp(X, Y)
    R2, t2 = cesa.emicp(X, Y)
    assert np.array_equal(R1, R2) and np.array_equal(t1, t2)  # deterministic
    dRt = torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    cesa.emicp_device(soa_tensor(torch, X), soa_tensor(torch, Y), dRt, d_status=st)
    torch.cuda.synchronize()
    assert int(st.item()) == 0 and cesa.stream_status() == 0
    out = dRt.cpu().numpy().astype(np.float64)
    assert np.array_equal(out[:9].reshape(3, 3), R1) and np.array_equal(out[9:], t1)


def test_c3_full_size_invariances(cesa):
    """N = M = 40,097 (config 3): size-independent properties of the result:
    permuting either cloud and moving the target rigidly leave the solution
    consistent (the FP64 oracle is too slow at this size)."""
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, Rt, tt = W.make("c3_emicp_40097", seed=0)
    R, t = cesa.emicp(X, Y)
    rng = np.random.default_rng(1)
    Rp, tp = cesa.emicp(X[rng.permutation(len(X))], Y[rng.permutation(len(Y))])
    assert rot_err_deg(Rp, R) < 1e-3
    assert np.abs(tp - t).max() < 1e-5 * float(np.ptp(X, 0).max())
    G = W.random_rotation(rng, 20.0)
    g = np.array([0.03, -0.01, 0.02])
    Xg = (X.astype(np.float64) @ G.T + g).astype(np.float32)
    Rg, tg = cesa.emicp(Xg, Y, G, g)
    # starting from the moved identity pose, the moved solution is G R, G t + g
    assert rot_err_deg(Rg, G @ R) < 2e-3
    assert np.abs(tg - (G @ t + g)).max() < 2e-5 * float(np.ptp(X, 0).max())
    # converged into the right basin (EM-ICP's own bias with 5% outliers and
    # partial overlap is about a degree here)
    assert rot_err_deg(R, Rt) < 3.0
