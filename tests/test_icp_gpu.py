"""ICP (cesa_icp / cesa_icp_device) on the GPU against the FP64 oracle's
restatement of src/icp.cpp:122-290 with exhaustive nearest neighbours.

The matches are discrete: FP32 and FP64 distances can order two nearly
equidistant candidates differently, so the match lists are compared as the
fraction that agree (at least 99.9%), and the pose within 1e-3 degrees and
1e-5 x the cloud extent (a flipped near-tie moves S by far less than that).
Equal distances go to the lowest X index in both.
"""
import numpy as np
import pytest

from conftest import rot_err_deg, soa_tensor

pytestmark = pytest.mark.gpu


def _check(R, t, Ro, to, X):
    extent = float(np.ptp(X, 0).max())
    assert np.all(np.isfinite(R)) and np.all(np.isfinite(t))
    assert rot_err_deg(R, Ro) < 1e-3, rot_err_deg(R, Ro)
    assert np.abs(t - to).max() < 1e-5 * extent, np.abs(t - to).max()


def _device_nn(cesa, torch, X, Y, p):
    dX, dY = soa_tensor(torch, X), soa_tensor(torch, Y)
    dRt = torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")
    nn = torch.full((len(Y),), -1, dtype=torch.int32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    cesa.icp_device(dX, dY, dRt, param=p, d_nn=nn, d_status=st)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    v = dRt.cpu().numpy().astype(np.float64)
    return v[:9].reshape(3, 3), v[9:], nn.cpu().numpy()


@pytest.mark.parametrize("gen,n,seed", [("uniform", 1007, 0), ("surface", 2000, 1), ("uniform", 8000, 2)])
def test_icp_matches_oracle(cesa, oracle, torch_cuda, gen, n, seed):
    from cuda_emicp_softassign_gb300 import workloads as W
    if gen == "uniform":
        X, Y, _, _ = W.uniform_pair(n=n, seed=seed, max_deg=20.0, t_range=0.05)
    else:
        X, Y, _, _ = W.surface_pair(n=n, seed=seed)
    iters = 30 if n <= 2000 else 10
    p = cesa.Params.default(maxIteration=iters)
    R, t, tr, rep = cesa.icp(X, Y, param=p, trace=True)
    Ro, to, tro, nno = oracle.icp(X, Y, maxIteration=iters)
    _check(R, t, Ro, to, X)
    assert rep.steps == iters and len(tr) == iters
    # per-iteration cost (sum of squared match distances) and centres
    assert np.allclose(tr[:, 2], tro[:, 2], rtol=1e-4)
    assert np.abs(tr[:, 3:9] - tro[:, 3:9]).max() < 1e-5
    Rd, td, nn = _device_nn(cesa, torch_cuda, X, Y, p)
    assert np.array_equal(Rd, R) and np.array_equal(td, t)
    assert np.mean(nn == nno) >= 0.999


@pytest.mark.parametrize("n,m", [(1, 1), (2, 5), (1, 300), (300, 1), (1025, 3000), (3001, 1023)])
def test_icp_ragged_and_tiny(cesa, oracle, torch_cuda, n, m):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.uniform_pair(n=n, m=m, seed=n + 7 * m, max_deg=10.0, t_range=0.03)
    p = cesa.Params.default(maxIteration=8)
    Rd, td, nn = _device_nn(cesa, torch_cuda, X, Y, p)
    Ro, to, _, nno = oracle.icp(X, Y, maxIteration=8)
    assert np.all(np.isfinite(Rd)) and np.all(np.isfinite(td))
    assert np.allclose(Rd @ Rd.T, np.eye(3), atol=1e-5)
    assert nn.min() >= 0 and nn.max() < n
    if min(n, m) >= 100:  # S is (near) degenerate for a handful of points
        _check(Rd, td, Ro, to, X)
        assert np.mean(nn == nno) >= 0.999


def test_icp_equal_distances_take_the_lowest_index(cesa, torch_cuda):
    """Duplicate target points: every match is the first copy."""
    rng = np.random.default_rng(3)
    base = rng.uniform(0, 1, (300, 3))
    X = np.concatenate([base, base, base])  # index i, i + 300, i + 600 are the same point
    Y = base[rng.permutation(300)]
    _, _, nn = _device_nn(cesa, torch_cuda, X, Y, cesa.Params.default(maxIteration=3))
    assert nn.max() < 300


def test_icp_deterministic_and_zero_iterations(cesa):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.uniform_pair(n=3000, seed=9, max_deg=15.0, t_range=0.05)
    p = cesa.Params.default(maxIteration=12)
    R1, t1 = cesa.icp(X, Y, param=p)
    R2, t2 = cesa.icp(X, Y, param=p)
    assert np.array_equal(R1, R2) and np.array_equal(t1, t2)
    R0 = np.array([[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    R, t = cesa.icp(X, Y, R0, np.array([0.1, 0.2, 0.3]), param=cesa.Params.default(maxIteration=0))
    assert np.allclose(R, R0) and np.allclose(t, [0.1, 0.2, 0.3], atol=1e-6)


@pytest.mark.parametrize("n,m,seed", [(5000, 4000, 21), (20000, 3000, 22), (300, 2000, 23)])
def test_grid_search_equals_exhaustive_bitwise(cesa, torch_cuda, n, m, seed):
    """The grid search returns the same matches as the exhaustive search (both
    take the first of equal distances), so the registrations are bitwise equal;
    surface views (a 2-D manifold in a 3-D grid) and a uniform cube."""
    from cuda_emicp_softassign_gb300 import workloads as W
    if seed == 21:
        X, Y, _, _ = W.uniform_pair(n=n, m=m, seed=seed, max_deg=20.0, t_range=0.05)
    else:
        X, Y, _, _ = W.surface_pair(n=n, m=m, seed=seed)
    out = []
    for mode in (cesa.ICP_SEARCH_EXHAUSTIVE, cesa.ICP_SEARCH_GRID):
        p = cesa.Params.default(maxIteration=12, icp_search=mode)
        out.append(_device_nn(cesa, torch_cuda, X, Y, p))
    (R1, t1, nn1), (R2, t2, nn2) = out
    assert np.array_equal(nn1, nn2)
    assert np.array_equal(R1, R2) and np.array_equal(t1, t2)


def test_grid_search_far_points_and_duplicates(cesa, torch_cuda):
    """Queries far outside the target's grid, duplicate targets (equal
    distances: the lowest index) and a flat target (one-cell-thick grid)."""
    rng = np.random.default_rng(4)
    base = rng.uniform(0, 1, (2500, 3))
    base[:, 2] = 0.0  # flat
    X = np.concatenate([base, base])
    Y = np.concatenate([base[rng.permutation(2500)][:2000], rng.uniform(-50, 50, (300, 3))])
    res = []
    for mode in (cesa.ICP_SEARCH_EXHAUSTIVE, cesa.ICP_SEARCH_GRID):
        res.append(_device_nn(cesa, torch_cuda, X, Y, cesa.Params.default(maxIteration=1, icp_search=mode)))
    assert np.array_equal(res[0][2], res[1][2])
    assert res[1][2][:2000].max() < 2500
