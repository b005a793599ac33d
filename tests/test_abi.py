"""C ABI of libcesa.so without a GPU: exports, layouts, host-side functions,
argument checks and the loud failure when no device is present."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import REPO, rot_err_deg

HEADER = os.path.join(REPO, "include", "cesa.h")
GOLD = os.path.join(REPO, "tests", "golden")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cesa_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(cesa):
    names = declared_functions()
    assert len(names) >= 12
    L = cesa.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", cesa.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (\w+)", out))
    assert set(names) <= exported
    assert all(n.startswith("cesa_") for n in exported), "only cesa_* may be exported"


def _c_layout(code, extra_inc=()):
    d = tempfile.mkdtemp()
    src = os.path.join(d, "l.cpp")
    exe = os.path.join(d, "l")
    open(src, "w").write(code)
    cmd = ["g++", "-std=c++17", "-I", os.path.join(REPO, "include")]
    for inc in extra_inc:
        cmd += ["-I", inc]
    subprocess.run(cmd + [src, "-o", exe], check=True)
    return subprocess.run([exe], capture_output=True, text=True, check=True).stdout


def test_params_mirror_matches_c_layout(cesa):
    code = r'''
#include <cstdio>
#include <cstddef>
#include "cesa.h"
#define F(x) printf("%s %zu\n", #x, offsetof(cesa_params, x));
int main(){ printf("size %zu\n", sizeof(cesa_params));
F(JMAX)F(I0)F(I1)F(alpha)F(T_0)F(TFACTOR)F(moutlier)F(sigma_p2)F(sigma_inf)F(sigma_factor)F(d_02)
F(maxIteration)F(sinkhorn_form)F(timeout_ms)F(device)F(icp_search)F(emicp_backward_layout)F(softassign_backward_form)F(reserved)
printf("report %zu\n", sizeof(cesa_report));
printf("pair %zu\n", sizeof(cesa_pair));
printf("pair_params %zu\n", offsetof(cesa_pair, params));
printf("pair_Rt %zu\n", offsetof(cesa_pair, Rt)); }
'''
    got = dict(l.split() for l in _c_layout(code).strip().splitlines())
    P = cesa.Params
    assert int(got["size"]) == ctypes.sizeof(P)
    for name, _ in P._fields_:
        if name in got:
            assert int(got[name]) == getattr(P, name).offset, name
    assert int(got["report"]) == ctypes.sizeof(cesa.Report)
    assert int(got["pair"]) == ctypes.sizeof(cesa.Pair)
    assert int(got["pair_params"]) == cesa.Pair.params.offset
    assert int(got["pair_Rt"]) == cesa.Pair.Rt.offset


def test_registration_parameters_layout_matches_reference():
    """include/3dregistration.h keeps the reference's registrationParameters
    field order and offsets (src/3dregistration.h:39-76)."""
    from oracle import build as ob
    ref_src = ob.reference_sources()  # the reference tree, or the copies staged from it
    if ref_src is None:
        pytest.skip("reference sources not available")
    fields = ["JMAX", "I0", "I1", "alpha", "T_0", "TFACTOR", "moutlier", "sigma_p2", "sigma_inf",
              "sigma_factor", "d_02", "maxIteration", "noviewer", "nostop", "notimer", "argc", "argv",
              "viewer", "source_trans_color", "cloud_source", "cloud_source_trans", "cloud_target"]
    body = "".join('printf("%%s %%zu\\n", "%s", offsetof(registrationParameters, %s));' % (f, f) for f in fields)
    code = '#include <cstdio>\n#include <cstddef>\n#include "3dregistration.h"\nint main(){%s printf("size %%zu\\n", sizeof(registrationParameters));}\n' % body
    ours = _c_layout(code.replace("3dregistration.h", os.path.join(REPO, "include", "3dregistration.h")))
    theirs = _c_layout(code.replace("3dregistration.h", os.path.join(ref_src, "3dregistration.h")),
                       extra_inc=[os.path.join(REPO, "oracle", "stubs")])
    assert ours == theirs


def test_params_defaults_are_reference_cli_defaults(cesa):
    p = cesa.Params.default()
    assert (p.JMAX, p.I0, p.I1) == (100, 5, 3)
    assert p.alpha == pytest.approx(3.0) and p.T_0 == pytest.approx(100.0)
    assert p.TFACTOR == pytest.approx(0.95)
    assert p.moutlier == pytest.approx(np.exp(-1.0) / 10.0, rel=1e-6)
    assert p.sigma_p2 == np.float32(0.01) and p.sigma_inf == np.float32(1e-5)
    assert p.sigma_factor == np.float32(0.9) and p.d_02 == np.float32(0.01)
    assert p.maxIteration == 30 and p.device == -1


def test_find_rt_from_s_matches_reference_golden(cesa, oracle):
    g = np.load(os.path.join(GOLD, "findrt_reference.npz"))
    for k in range(len(g["S"])):
        R, t = cesa.find_rt_from_s(g["Xc"][k], g["Yc"][k], g["S"][k])
        _, _, info = oracle.find_rt_from_s(g["Xc"][k], g["Yc"][k], g["S"][k])
        if info["gap"] > 1e-3:
            assert rot_err_deg(R, g["R"][k]) < 1e-3, k
            assert np.abs(t - g["t"][k]).max() < 1e-4 * (1 + np.abs(g["t"][k]).max()), k


def test_find_rt_from_s_fallback_keeps_previous_quaternion(cesa):
    q = np.array([np.cos(0.3), 0.0, np.sin(0.3), 0.0], np.float32)
    R, t = cesa.find_rt_from_s(np.zeros(3), np.ones(3), np.full(9, np.nan), q_prev=q)
    assert abs(R[1, 1] - 1.0) < 1e-6 and abs(R[0, 0] - np.cos(0.6)) < 1e-6


def test_cloud2data_is_soa(cesa):
    P = np.arange(15, dtype=np.float32).reshape(5, 3)
    assert np.array_equal(cesa.cloud2data(P), P.T.reshape(-1))
    P4 = np.c_[P, np.ones(5, np.float32)]  # PCL-style padded points
    assert np.array_equal(cesa.cloud2data(P4), P.T.reshape(-1))


def test_invalid_arguments_are_rejected(cesa):
    L = cesa.lib()
    X = np.zeros(6, np.float32)
    R = np.eye(3, dtype=np.float32).reshape(-1)
    t = np.zeros(3, np.float32)
    p = cesa.Params.default()
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    assert L.cesa_emicp(ptr(X), 0, ptr(X), 2, ptr(R), ptr(t), ctypes.byref(p), None) == cesa.CESA_ERR_INVALID_ARGUMENT
    assert L.cesa_emicp(None, 2, ptr(X), 2, ptr(R), ptr(t), ctypes.byref(p), None) == cesa.CESA_ERR_INVALID_ARGUMENT
    bad = cesa.Params.default(sigma_factor=1.5)  # would never terminate in the reference
    assert L.cesa_emicp(ptr(X), 2, ptr(X), 2, ptr(R), ptr(t), ctypes.byref(bad), None) == cesa.CESA_ERR_INVALID_ARGUMENT
    bad = cesa.Params.default(I1=0)  # the reference would read uninitialised column sums
    assert L.cesa_softassign(ptr(X), 2, ptr(X), 2, ptr(R), ptr(t), ctypes.byref(bad), None) == cesa.CESA_ERR_INVALID_ARGUMENT
    assert cesa.status_string(cesa.CESA_ERR_TIMEOUT) == "device-side wait timed out"
    # ICP and the adjoints validate before touching a device
    assert L.cesa_icp(ptr(X), 2, ptr(X), 0, ptr(R), ptr(t), ctypes.byref(p), None) == cesa.CESA_ERR_INVALID_ARGUMENT
    bad = cesa.Params.default(maxIteration=-1)
    assert L.cesa_icp(ptr(X), 2, ptr(X), 2, ptr(R), ptr(t), ctypes.byref(bad), None) == cesa.CESA_ERR_INVALID_ARGUMENT
    assert L.cesa_softassign_tape_bytes(0, 5, ctypes.byref(p)) == 0
    assert L.cesa_softassign_tape_bytes(5, 5, ctypes.byref(cesa.Params.default(I1=0))) == 0
    assert L.cesa_emicp_tape_bytes(5, 0, ctypes.byref(p)) == 0
    assert L.cesa_softassign_backward_device(5, 5, ctypes.byref(p), None, None, None, None, None, None, None) == \
        cesa.CESA_ERR_INVALID_ARGUMENT
    assert L.cesa_emicp_backward_device(0, 5, ctypes.byref(p), None, None, None, None, None, None, None) == \
        cesa.CESA_ERR_INVALID_ARGUMENT
    # out-of-range execution controls (the pointers are checked for NULL only, never read)
    d = ptr(X)
    bad = cesa.Params.default(emicp_backward_layout=cesa.LAYOUT_RANGED + 1)
    assert L.cesa_emicp_backward_device(5, 5, ctypes.byref(bad), d, d, d, d, d, None, None) == \
        cesa.CESA_ERR_INVALID_ARGUMENT
    bad = cesa.Params.default(softassign_backward_form=-1)
    assert L.cesa_softassign_backward_device(5, 5, ctypes.byref(bad), d, d, d, d, d, None, None) == \
        cesa.CESA_ERR_INVALID_ARGUMENT
    assert cesa.status_string(cesa.CESA_ERR_INTERNAL).startswith("internal consistency check failed")


def test_tape_sizes_grow_with_the_schedule(cesa):
    """The Softassign tape holds, per pose update, the record, the slack and
    4 (N + M) floats per Sinkhorn pass plus 5 N; EM-ICP's, per sigma step, the
    record and 5 M floats."""
    L = cesa.lib()
    p = cesa.Params.default(JMAX=10, I0=5, I1=3)
    n = L.cesa_softassign_tape_bytes(1000, 800, ctypes.byref(p))
    per_update = 4 * (64 + 1000 + 800 + 3 * 4 * (1000 + 800) + 5 * 1000)
    assert per_update * 50 <= n <= per_update * 50 + 4 * 256 * 12 + 16 * (1000 + 800) + 256
    q = cesa.Params.default(JMAX=20, I0=5, I1=3)
    # 50 more updates: the same per-update bytes again, up to the sections' 256-byte alignment
    assert abs(L.cesa_softassign_tape_bytes(1000, 800, ctypes.byref(q)) - n - per_update * 50) <= 6 * 256


def test_invalid_batches_are_rejected(cesa):
    L = cesa.lib()
    X = np.zeros(6, np.float32)
    rt = np.zeros(12, np.float32)
    arr = (cesa.Pair * 2)()
    for k in range(2):
        arr[k].algorithm = cesa.ALGO_EMICP
        arr[k].N = arr[k].M = 2
        arr[k].X = arr[k].Y = X.ctypes.data
        arr[k].Rt = rt.ctypes.data
        arr[k].params = cesa.Params.default()
    call = lambda n: L.cesa_register_batch(ctypes.cast(arr, ctypes.c_void_p), n, None)  # noqa: E731
    assert call(0) == cesa.CESA_ERR_INVALID_ARGUMENT
    arr[1].algorithm = 7
    assert call(2) == cesa.CESA_ERR_INVALID_ARGUMENT
    arr[1].algorithm = cesa.ALGO_SOFTASSIGN
    arr[1].params = cesa.Params.default(I1=0)
    assert call(2) == cesa.CESA_ERR_INVALID_ARGUMENT
    arr[1].params = cesa.Params.default()
    arr[1].M = 0
    assert call(2) == cesa.CESA_ERR_INVALID_ARGUMENT
    assert L.cesa_register_batch(None, 1, None) == cesa.CESA_ERR_INVALID_ARGUMENT
    assert L.cesa_register_batch_device(ctypes.cast(arr, ctypes.c_void_p), cesa.MAX_BATCH + 1, None,
                                        None) == cesa.CESA_ERR_INVALID_ARGUMENT


def test_no_cpu_fallback_without_gpu(cesa):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    X = np.random.default_rng(0).uniform(0, 1, (20, 3)).astype(np.float32)
    with pytest.raises(cesa.CesaError) as e:
        cesa.emicp(X, X)
    assert e.value.code == cesa.CESA_ERR_NO_DEVICE
    with pytest.raises(cesa.CesaError):
        cesa.softassign(X, X)


@pytest.fixture(scope="module")
def pose_harness():
    d = tempfile.mkdtemp()
    so = os.path.join(d, "pose.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I",
                    os.path.join(REPO, "cuda_emicp_softassign_gb300", "csrc"),
                    os.path.join(REPO, "tests", "pose_harness.cpp"), "-o", so], check=True)
    return ctypes.CDLL(so)


def _quat_R(q):
    q0, qx, qy, qz = q
    return np.array([[q0*q0+qx*qx-qy*qy-qz*qz, 2*(qx*qy-q0*qz), 2*(qx*qz+q0*qy)],
                     [2*(qy*qx+q0*qz), q0*q0-qx*qx+qy*qy-qz*qz, 2*(qy*qz-q0*qx)],
                     [2*(qz*qx-q0*qy), 2*(qz*qy+q0*qx), q0*q0-qx*qx-qy*qy+qz*qz]])


def test_device_pose_solver_fp32_warm_start(pose_harness, oracle):
    """The FP32 warm-started Jacobi used on the device, run on the host over an
    annealing-like sequence of slowly rotating S, against the FP64 oracle."""
    from cuda_emicp_softassign_gb300 import workloads as W
    rng = np.random.default_rng(9)
    K = 200
    base = rng.standard_normal((3, 3)) * 0.05
    Ss = []
    for k in range(K):
        A = W._rot([1.0, 2.0, 0.5], np.radians(40.0 * k / K))
        S = A * (1.0 + 0.3 * np.sin(k / 7.0)) + base
        Ss.append(S.reshape(-1, order="F"))
    S32 = np.ascontiguousarray(np.array(Ss, np.float32))
    q = np.zeros((K, 4), np.float32)
    gap = np.zeros(K, np.float32)
    fb = pose_harness.pose_sequence_f32(S32.ctypes.data_as(ctypes.c_void_p), K,
                                        q.ctypes.data_as(ctypes.c_void_p), gap.ctypes.data_as(ctypes.c_void_p))
    assert fb == 0
    worst = 0.0
    for k in range(K):
        Ro, _, info = oracle.find_rt_from_s(np.zeros(3), np.zeros(3), S32[k].astype(np.float64))
        e = rot_err_deg(_quat_R(q[k].astype(np.float64)), Ro)
        worst = max(worst, e)
        assert abs(gap[k] - info["gap"]) < 1e-4 * max(1.0, info["gap"])
    assert worst < 1e-4, worst


def _fast_sequence(pose_harness, S32):
    K = len(S32)
    q = np.zeros((K, 4), np.float32)
    lmax = np.zeros(K, np.float32)
    jac = pose_harness.pose_sequence_fast_f32(np.ascontiguousarray(S32).ctypes.data_as(ctypes.c_void_p), K,
                                              q.ctypes.data_as(ctypes.c_void_p), lmax.ctypes.data_as(ctypes.c_void_p))
    return q, lmax, jac


def test_fast_pose_solver_warm_sequence(pose_harness, oracle):
    """The plain kernels' solver (certified shifted inverse iteration from the
    previous quaternion, Jacobi fallback) over the same annealing-like
    sequence: as accurate as the Jacobi path, and it falls back only where the
    previous quaternion is far (the first solve)."""
    from cuda_emicp_softassign_gb300 import workloads as W
    rng = np.random.default_rng(9)
    K = 200
    base = rng.standard_normal((3, 3)) * 0.05
    S32 = np.array([(W._rot([1.0, 2.0, 0.5], np.radians(40.0 * k / K)) * (1.0 + 0.3 * np.sin(k / 7.0)) + base)
                    .reshape(-1, order="F") for k in range(K)], np.float32)
    q, lmax, jac = _fast_sequence(pose_harness, S32)
    assert jac <= 2, jac
    worst = 0.0
    for k in range(K):
        Ro, _, info = oracle.find_rt_from_s(np.zeros(3), np.zeros(3), S32[k].astype(np.float64))
        worst = max(worst, rot_err_deg(_quat_R(q[k].astype(np.float64)), Ro))
    assert worst < 1e-4, worst


def test_fast_pose_solver_refuses_what_it_cannot_certify(pose_harness, oracle):
    """Jumps of 90 degrees between solves and near-degenerate top eigenvalues
    (S = diag(1, 0.2, -0.2): N = diag(1, 1, -0.6, -1.4), plus 1e-7 noise) are
    refused by the inverse iteration and solved by the Jacobi fallback, still
    matching the FP64 oracle wherever its own gap is resolvable."""
    from cuda_emicp_softassign_gb300 import workloads as W
    rng = np.random.default_rng(11)
    jumps = np.array([W._rot(rng.standard_normal(3), np.radians(90.0 * (k % 2))).reshape(-1, order="F")
                      for k in range(20)], np.float32)
    q, _, jac = _fast_sequence(pose_harness, jumps)
    assert jac >= 10, jac
    for k in range(20):
        Ro, _, _ = oracle.find_rt_from_s(np.zeros(3), np.zeros(3), jumps[k].astype(np.float64))
        assert rot_err_deg(_quat_R(q[k].astype(np.float64)), Ro) < 1e-3
    near = []
    for k in range(20):
        A = np.diag([1.0, 0.2, -0.2]) + 1e-7 * rng.standard_normal((3, 3))
        near.append(A.reshape(-1, order="F"))
    near = np.array(near, np.float32)
    q, _, jac = _fast_sequence(pose_harness, near)
    assert jac == 20, jac


def test_device_pose_solver_random_cold(pose_harness, oracle):
    rng = np.random.default_rng(10)
    for _ in range(100):
        S = rng.standard_normal(9)
        q = np.zeros(4)
        gap = np.zeros(1)
        pose_harness.pose_sequence_f64(np.ascontiguousarray(S).ctypes.data_as(ctypes.c_void_p), 1,
                                       q.ctypes.data_as(ctypes.c_void_p), gap.ctypes.data_as(ctypes.c_void_p))
        Ro, _, info = oracle.find_rt_from_s(np.zeros(3), np.zeros(3), S)
        if info["gap"] > 1e-6:
            assert rot_err_deg(_quat_R(q), Ro) < 1e-7


def test_device_pose_solvers_along_config_trajectories(pose_harness, oracle):
    """Both FP32 pose solves of the kernels -- the warm-started Jacobi (taped
    and matrix-free kernels) and the certified inverse iteration with its
    Jacobi fallback (EM-ICP, banded Softassign, ICP) -- along the S sequences
    of whole registrations: config 3's 66 EM-ICP steps and config 2's 500
    Softassign updates, from the FP64 oracle's stored traces. Against the
    FP64 solve of each S: within 1e-4 degrees per step wherever Horn's
    relative eigen-gap exceeds 1e-3 (every step of both sequences here), and
    the gap itself within 1e-4."""
    for name in ("c3_emicp_40097.npz", "c2_softassign_2000.npz"):
        g = np.load(os.path.join(GOLD, name))
        S32 = np.ascontiguousarray(g["trace"][:, 9:18].astype(np.float32))
        K = len(S32)
        qj = np.zeros((K, 4), np.float32)
        gap = np.zeros(K, np.float32)
        pose_harness.pose_sequence_f32(S32.ctypes.data_as(ctypes.c_void_p), K, qj.ctypes.data_as(ctypes.c_void_p),
                                       gap.ctypes.data_as(ctypes.c_void_p))
        qf, _, _ = _fast_sequence(pose_harness, S32)
        worst_j = worst_f = 0.0
        for k in range(K):
            Ro, _, info = oracle.find_rt_from_s(np.zeros(3), np.zeros(3), S32[k].astype(np.float64))
            assert info["gap"] > 1e-3, (name, k, info["gap"])
            e_j = rot_err_deg(_quat_R(qj[k].astype(np.float64)), Ro)
            e_f = rot_err_deg(_quat_R(qf[k].astype(np.float64)), Ro)
            assert e_j < 1e-4 and e_f < 1e-4, (name, k, e_j, e_f, info["gap"])
            assert abs(gap[k] - info["gap"]) < 1e-4 * max(1.0, info["gap"]), (name, k)
            worst_j, worst_f = max(worst_j, e_j), max(worst_f, e_f)
        print("%s: %d solves, worst %.2e deg (Jacobi), %.2e deg (certified)" % (name, K, worst_j, worst_f))
