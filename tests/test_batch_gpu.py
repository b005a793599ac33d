"""Batched registration (cesa_register_batch*) on the GPU, against the FP64
oracle and against the single-pair entry points.

Every pair of a batch must meet the single-pair criteria: EM-ICP within 1e-3
degrees and 1e-5 x extent of the FP64 oracle; Softassign within max(1e-3 deg,
0.25 x the error of the reference's own FP32 arithmetic) over the default
schedule. Each pair's sums run in a fixed order whatever block runs them, so
a pair's result does not depend on where it sits in the batch (bitwise). The
slice length of the (pair, tile) units follows the batch's total work, so the
same pair in a different batch agrees to rounding.
"""
import numpy as np
import pytest

from conftest import rot_err_deg, soa_tensor

pytestmark = pytest.mark.gpu


def _mixed_pairs():
    from cuda_emicp_softassign_gb300 import workloads as W
    pairs = []
    for n, m, seed in ((300, 280, 1), (1200, 700, 2), (64, 900, 3), (1500, 1500, 4)):
        X, Y, _, _ = W.uniform_pair(n=n, m=m, seed=seed, max_deg=20.0, t_range=0.05)
        pairs.append(("emicp", X, Y))
    for n, m, seed in ((200, 200, 1), (160, 240, 2), (333, 100, 3)):
        X, Y, _, _ = W.surface_pair(n=n, m=m, seed=seed)
        pairs.append(("softassign", X, Y))
    return pairs


def _batch_args(cesa, pairs):
    out = []
    for kind, X, Y in pairs:
        algo = cesa.ALGO_EMICP if kind == "emicp" else cesa.ALGO_SOFTASSIGN
        out.append((algo, X, Y, cesa.Params.default()))
    return out


@pytest.fixture(scope="module")
def mixed(cesa):
    pairs = _mixed_pairs()
    res, rep = cesa.register_batch(_batch_args(cesa, pairs), report=True)
    return pairs, res, rep


def test_mixed_batch_matches_oracle(cesa, oracle, mixed):
    pairs, res, rep = mixed
    assert rep.steps == 8 * 500  # the Softassign schedule is the longest: (2 I1 + 2) x JMAX x I0 rounds
    for (kind, X, Y), (R, t) in zip(pairs, res):
        extent = float(np.ptp(X, 0).max())
        assert np.all(np.isfinite(R)) and np.all(np.isfinite(t))
        if kind == "emicp":
            Ro, to, _ = oracle.emicp(X, Y)
            assert rot_err_deg(R, Ro) < 1e-3, (len(X), len(Y))
            assert np.abs(t - to).max() < 1e-5 * extent, (len(X), len(Y))
        else:
            Ro, to, _ = oracle.softassign(X, Y)
            Rp, tp, _ = oracle.softassign(X, Y, precision="f32", trace=False)
            e, e_port = rot_err_deg(R, Ro), rot_err_deg(Rp, Ro)
            assert e <= max(1e-3, 0.25 * e_port), (len(X), len(Y), e, e_port)
            assert np.abs(t - to).max() <= max(1e-5 * extent, 0.25 * np.abs(tp - to).max())


def test_mixed_batch_agrees_with_single_pair_calls(cesa, mixed):
    pairs, res, _ = mixed
    for (kind, X, Y), (R, t) in zip(pairs, res):
        Rs, ts = (cesa.emicp if kind == "emicp" else cesa.softassign)(X, Y)
        extent = float(np.ptp(X, 0).max())
        tol = 1e-4 if kind == "emicp" else 2e-3
        assert rot_err_deg(R, Rs) < tol, (kind, len(X), len(Y))
        assert np.abs(t - ts).max() < (1e-5 if kind == "emicp" else 1e-4) * extent


def test_pair_result_is_independent_of_the_batch_order(cesa, mixed):
    """Bitwise under reversal and rotation of the pair order; a pair alone in
    a batch of one agrees to rounding."""
    pairs, res, _ = mixed
    args = _batch_args(cesa, pairs)
    rev = cesa.register_batch(args[::-1])[::-1]
    for (R, t), (Rr, tr) in zip(res, rev):
        assert np.array_equal(R, Rr) and np.array_equal(t, tr)
    rot = cesa.register_batch(args[3:] + args[:3])
    rot = rot[-3:] + rot[:-3]
    for (R, t), (Rr, tr) in zip(res, rot):
        assert np.array_equal(R, Rr) and np.array_equal(t, tr)
    (R1, t1), = cesa.register_batch([args[0]])
    assert rot_err_deg(R1, res[0][0]) < 1e-4


def test_device_entry_point_matches_host(cesa, torch_cuda, mixed):
    torch = torch_cuda
    pairs, res, _ = mixed
    dev = []
    keep = []
    for (kind, X, Y), (_, _, _, p) in zip(pairs, _batch_args(cesa, pairs)):
        dX, dY = soa_tensor(torch, X), soa_tensor(torch, Y)
        dRt = torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")
        algo = cesa.ALGO_EMICP if kind == "emicp" else cesa.ALGO_SOFTASSIGN
        dev.append((algo, dX, dY, dRt, p))
        keep.append(dRt)
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    cesa.register_batch_device(dev, d_status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    assert cesa.stream_status() == 0
    for dRt, (R, t) in zip(keep, res):
        v = dRt.cpu().numpy()
        assert np.array_equal(v[:9].reshape(3, 3).astype(np.float64), R)
        assert np.array_equal(v[9:].astype(np.float64), t)


def test_ragged_and_tiny_pairs(cesa, oracle):
    from cuda_emicp_softassign_gb300 import workloads as W
    sizes = [(1, 1), (2, 3), (129, 1), (1, 500), (513, 200), (127, 129)]
    pairs = []
    for i, (n, m) in enumerate(sizes):
        X, Y, _, _ = W.uniform_pair(n=n, m=m, seed=10 + i, max_deg=10.0, t_range=0.03)
        pairs.append((cesa.ALGO_EMICP, X, Y, cesa.Params.default(sigma_inf=2e-4)))
        pairs.append((cesa.ALGO_SOFTASSIGN, X, Y, cesa.Params.default(JMAX=4)))
    res = cesa.register_batch(pairs)
    for (algo, X, Y, _), (R, t) in zip(pairs, res):
        n, m = len(X), len(Y)
        if algo == cesa.ALGO_EMICP:
            Ro, to, _ = oracle.emicp(X, Y, sigma_inf=2e-4)
        else:
            Ro, to, _ = oracle.softassign(X, Y, JMAX=4)
        # With a single X point the reference's Softassign drains the
        # assignment into the slack: sumM -> 0 while its Y centre, sum cs y /
        # sumM, grows until t overflows to NaN (the FP64 oracle too).
        # Finiteness is required wherever the oracle's result is finite.
        assert np.all(np.isfinite(R)), (algo, n, m)
        assert np.array_equal(np.isfinite(t), np.isfinite(to)), (algo, n, m, t, to)
        assert np.allclose(R @ R.T, np.eye(3), atol=1e-5)
        if min(n, m) < 100:
            continue  # S is (near) degenerate: R is not determined
        if algo == cesa.ALGO_EMICP:
            assert rot_err_deg(R, Ro) < 1e-3, (n, m)
        else:
            Rp, _, _ = oracle.softassign(X, Y, JMAX=4, precision="f32", trace=False)
            e, e_port = rot_err_deg(R, Ro), rot_err_deg(Rp, Ro)
            assert e <= max(1e-3, 2.0 * e_port), (n, m, e, e_port)
