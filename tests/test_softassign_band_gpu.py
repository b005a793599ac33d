"""Softassign with the banded Sinkhorn form (matrix-free arithmetic, one
thread-block cluster per band of 64 rows, row passes reduced through
distributed shared memory), against the FP64 oracle and the grid-wide
matrix-free form.

Only the summation orders differ from the matrix-free form. Tolerances are
those of the matrix-free tests: slack vectors and row/column sums 1e-5
relative; S relative to its largest entry within max(1e-5, 2x the
reference's own FP32 error); final R within max(1e-3 deg, 0.25x the FP32
port's error) over the default schedule.
"""
import numpy as np
import pytest

from conftest import rel_err, rot_err_deg, soa_tensor

pytestmark = pytest.mark.gpu


# every cluster size (1, 2, 4, 8 column tiles), ragged bands and tiles; 4100 x 60:
# 65 bands of one CTA (more than 32 band partials per column, 64 active rows in
# the moment sum)
@pytest.mark.parametrize("n,m", [(300, 300), (257, 129), (77, 500), (1000, 31), (130, 100), (600, 2048),
                                 (2000, 1100), (2000, 2000), (4100, 60)])
@pytest.mark.parametrize("T", [100.0, 0.7])
def test_inner_iteration_matches_oracle(cesa, oracle, torch_cuda, n, m, T):
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    X, Y, R, t = W.surface_pair(n=n, m=m, seed=n + 3 * m)
    mo = np.float32(0.0367879)
    s0 = np.full(n, mo * 0.7, np.float32)
    u0 = np.full(m, mo * 0.9, np.float32)
    ref = oracle.softassign_step(X, Y, R.astype(np.float32), t.astype(np.float32), T, 3.0, 3, s0, u0)
    s = torch.from_numpy(s0.copy()).cuda()
    u = torch.from_numpy(u0.copy()).cuda()
    rs = torch.zeros(n, device="cuda")
    cs = torch.zeros(m, device="cuda")
    w = torch.zeros(n, device="cuda")
    mom = cesa.softassign_step(soa_tensor(torch, X), soa_tensor(torch, Y), R, t, T, 3.0, 3, s, u,
                               rs=rs, cs=cs, w=w, form=cesa.SINKHORN_BANDED)
    torch.cuda.synchronize()
    for name, got in (("s", s), ("u", u), ("rs", rs), ("cs", cs), ("w", w)):
        g = got.cpu().numpy().astype(np.float64)
        assert np.all(np.abs(g - ref[name]) <= 1e-5 * np.abs(ref[name]) + 1e-30), name
    assert abs(mom[0] - ref["sum"]) <= 1e-5 * ref["sum"]
    port = oracle.softassign_step(X, Y, R.astype(np.float32), t.astype(np.float32), T, 3.0, 3, s0, u0,
                                  precision="f32")
    e_gpu, e_port = rel_err(mom[7:16], ref["S"]), rel_err(port["S"], ref["S"])
    assert e_gpu <= max(1e-5, 2.0 * e_port), (e_gpu, e_port)


@pytest.mark.parametrize("n,m,seed", [(200, 200, 1), (160, 240, 2), (333, 100, 3)])
def test_full_schedule_matches_oracle(cesa, oracle, n, m, seed):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.surface_pair(n=n, m=m, seed=seed)
    p = cesa.Params.default(sinkhorn_form=cesa.SINKHORN_BANDED)
    R, t, tr, rep = cesa.softassign(X, Y, param=p, trace=True)
    assert rep.sinkhorn_form == cesa.SINKHORN_BANDED
    assert rep.steps == 500 and len(tr) == 500
    Ro, to, tro = oracle.softassign(X, Y)
    Rp, tp, _ = oracle.softassign(X, Y, precision="f32", trace=False)
    e, e_port = rot_err_deg(R, Ro), rot_err_deg(Rp, Ro)
    assert e <= max(1e-3, 0.25 * e_port), (e, e_port)
    extent = float(np.ptp(X, 0).max())
    assert np.abs(t - to).max() <= max(1e-5 * extent, 0.25 * np.abs(tp - to).max())
    # the trace's temperature schedule and sumM follow the oracle's (records
    # of 32: step, T, sumM, ...)
    assert np.allclose(tr[:, 1], tro[:, 1], rtol=1e-6)
    assert np.allclose(tr[:3, 2], tro[:3, 2], rtol=1e-4)


def test_c2_full_size_matches_oracle_and_matrix_free(cesa, oracle):
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c2_softassign_2000", seed=0)
    p = cesa.Params.default(sinkhorn_form=cesa.SINKHORN_BANDED)
    R, t, _, rep = cesa.softassign(X, Y, param=p, trace=True)
    assert rep.sinkhorn_form == cesa.SINKHORN_BANDED
    Ro, to, _ = oracle.softassign(X, Y)
    assert rot_err_deg(R, Ro) < 1e-3
    assert np.abs(t - to).max() < 1e-5 * float(np.ptp(X, 0).max())
    Rf, tf = cesa.softassign(X, Y, param=cesa.Params.default(sinkhorn_form=cesa.SINKHORN_MATRIX_FREE))
    assert rot_err_deg(R, Rf) < 1e-3


def test_auto_uses_the_banded_form_where_it_fills_the_gpu(cesa):
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c2_softassign_2000", seed=0)
    _, _, _, rep = cesa.softassign(X, Y, param=cesa.Params.default(JMAX=2), trace=True)
    assert rep.sinkhorn_form == cesa.SINKHORN_BANDED
    # a small pair does not fill the GPU: the grid-wide matrix-free form
    X, Y, _, _ = W.surface_pair(n=200, m=200, seed=1)
    _, _, _, rep = cesa.softassign(X, Y, param=cesa.Params.default(JMAX=2), trace=True)
    assert rep.sinkhorn_form == cesa.SINKHORN_MATRIX_FREE


def test_too_many_columns_falls_back_to_matrix_free(cesa):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.surface_pair(n=300, m=2049, seed=4)
    p = cesa.Params.default(JMAX=3, sinkhorn_form=cesa.SINKHORN_BANDED)
    R, t, _, rep = cesa.softassign(X, Y, param=p, trace=True)
    assert rep.sinkhorn_form == cesa.SINKHORN_MATRIX_FREE
    Rf, tf = cesa.softassign(X, Y, param=cesa.Params.default(JMAX=3, sinkhorn_form=cesa.SINKHORN_MATRIX_FREE))
    assert np.array_equal(R, Rf) and np.array_equal(t, tf)


def test_ragged_sizes_are_orthonormal_and_finite_where_the_oracle_is(cesa, oracle):
    """With one X point the reference's own arithmetic ends in 0/0 (sumM
    decays to zero): t is NaN in the FP64 oracle too, and must be here."""
    from cuda_emicp_softassign_gb300 import workloads as W
    p = cesa.Params.default(JMAX=3, sinkhorn_form=cesa.SINKHORN_BANDED)
    for n, m in ((1, 1), (2, 3), (129, 33), (33, 129), (64, 256), (65, 257), (513, 1), (1, 2048), (2200, 1900),
                 (4100, 60)):
        X, Y, _, _ = W.uniform_pair(n=n, m=m, seed=n + m, max_deg=10.0, t_range=0.03)
        R, t, _, rep = cesa.softassign(X, Y, param=p, trace=True)
        assert rep.sinkhorn_form == cesa.SINKHORN_BANDED, (n, m)
        _, to, _ = oracle.softassign(X, Y, JMAX=3, trace=False)
        assert np.array_equal(np.isfinite(t), np.isfinite(to)), (n, m)
        assert np.all(np.isfinite(R)) and np.allclose(R @ R.T, np.eye(3), atol=1e-5), (n, m)


def test_device_entry_point_and_determinism(cesa, torch_cuda):
    from cuda_emicp_softassign_gb300 import workloads as W
    torch = torch_cuda
    X, Y, _, _ = W.surface_pair(n=1700, m=1500, seed=5)
    p = cesa.Params.default(JMAX=10, sinkhorn_form=cesa.SINKHORN_BANDED)
    R1, t1 = cesa.softassign(X, Y, param=p)
    R2, t2 = cesa.softassign(X, Y, param=p)
    assert np.array_equal(R1, R2) and np.array_equal(t1, t2)
    dRt = torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")
    cesa.softassign_device(soa_tensor(torch, X), soa_tensor(torch, Y), dRt, param=p)
    torch.cuda.synchronize()
    assert cesa.stream_status() == 0
    v = dRt.cpu().numpy().astype(np.float64)
    assert np.array_equal(v[:9].reshape(3, 3), R1) and np.array_equal(v[9:], t1)
