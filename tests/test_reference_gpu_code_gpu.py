"""The GPU kernels against the reference's own GPU code: softassign() and
emicp() of src/softassign.cu and src/emicp.cu, their CUDA kernels and cuBLAS
calls run on the host by oracle/emu (tests/golden/make_golden.py stores their
results and their own per-update Xc, Yc, S, R, t).

Both computations are FP32; the FP64 oracle (pinned to the same reference
outputs in tests/test_oracle.py) measures how far each lands. Per case and
Sinkhorn form:
  * the GPU's final pose within max(1e-3 degrees, 2x the reference's own
    distance) of the FP64 oracle's, t within max(1e-5, 2x) x cloud extent;
  * the worst relative error of S over the updates within max(1e-4, 2x the
    reference's own).
"""
import os

import numpy as np
import pytest

from conftest import rot_err_deg

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _srel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture(scope="module")
def sa_gold():
    return np.load(os.path.join(GOLD, "softassign_reference.npz"))


def _cases():
    g = np.load(os.path.join(GOLD, "softassign_reference.npz"))
    return [str(n) for n in g["names"]]


@pytest.mark.parametrize("form", ["matrix_free", "banded", "materialised"])
@pytest.mark.parametrize("name", _cases())
def test_softassign_against_reference_softassign_cu(cesa, oracle, sa_gold, name, form):
    g = sa_gold
    X, Y = g[name + "_X"], g[name + "_Y"]
    J, I0, I1, alpha, T_0, TF = g[name + "_sched"]
    sch = dict(JMAX=int(J), I0=int(I0), I1=int(I1), alpha=float(alpha), T_0=float(T_0), TFACTOR=float(TF))
    code = {"matrix_free": cesa.SINKHORN_MATRIX_FREE, "banded": cesa.SINKHORN_BANDED,
            "materialised": cesa.SINKHORN_MATERIALISED}[form]
    moutlier = float(np.float32(1.0 / np.sqrt(np.float32(T_0)) * np.exp(np.float32(-1.0))))
    p = cesa.Params.default(sinkhorn_form=code, moutlier=moutlier, **sch)
    R, t, tr, rep = cesa.softassign(X, Y, param=p, trace=True)
    Ro, to, tro = oracle.softassign(X, Y, **sch)
    ext = float(np.ptp(X, 0).max())
    e_gpu, e_ref = rot_err_deg(R, Ro), rot_err_deg(g[name + "_R"], Ro)
    et_gpu = np.abs(t - to).max() / ext
    et_ref = np.abs(g[name + "_t"] - to).max() / ext
    n = len(tro)
    assert len(tr) == n
    s_gpu = max(_srel(tr[k, 9:18], tro[k, 9:18]) for k in range(n))
    s_ref = max(_srel(g[name + "_trace"][k, 9:18], tro[k, 9:18]) for k in range(n))
    print("%s %s (form used %d): vs FP64 R %.2e deg (reference %.2e), t %.2e (%.2e), S %.2e (%.2e)"
          % (name, form, rep.sinkhorn_form, e_gpu, e_ref, et_gpu, et_ref, s_gpu, s_ref))
    assert e_gpu <= max(1e-3, 2.0 * e_ref), (e_gpu, e_ref)
    assert et_gpu <= max(1e-5, 2.0 * et_ref), (et_gpu, et_ref)
    assert s_gpu <= max(1e-4, 2.0 * s_ref), (s_gpu, s_ref)


def test_emicp_against_reference_emicp_cu(cesa, oracle):
    """The fused EM-ICP kernel against the reference's GPU emicp() results:
    within 1e-3 degrees / 1e-5 x extent of them, and of the FP64 oracle."""
    g = np.load(os.path.join(GOLD, "emicp_gpu_reference.npz"))
    for name in g["names"]:
        name = str(name)
        X, Y = g[name + "_X"], g[name + "_Y"]
        R, t, tr, rep = cesa.emicp(X, Y, trace=True)
        ext = float(np.ptp(X, 0).max())
        assert rot_err_deg(R, g[name + "_R"]) < 1e-3, name
        assert np.abs(t - g[name + "_t"]).max() < 1e-5 * ext, name
        trr = g[name + "_trace"]
        for k in range(len(trr)):
            assert rot_err_deg(tr[k, 18:27].reshape(3, 3), trr[k, 18:27].reshape(3, 3)) < 1e-3, (name, k)
