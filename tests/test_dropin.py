"""The C++ drop-in boundary: a program written against the reference API
(3dregistration.h + registration.cpp, linked to libcesa.so), as the reference
README asks users to build with emicp.cu / softassign.cu."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import REPO, rot_err_deg


@pytest.fixture(scope="module")
def dropin_exe(cesa):
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "dropin")
    libdir = os.path.dirname(cesa.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "dropin_main.cpp"),
                    os.path.join(REPO, "cuda_emicp_softassign_gb300", "csrc", "registration.cpp"),
                    "-L", libdir, "-lcesa", "-Wl,-rpath," + libdir, "-o", exe], check=True)
    return exe


def _write(path, P):
    with open(path, "wb") as f:
        np.array([len(P)], np.int32).tofile(f)
        np.ascontiguousarray(P, np.float32).tofile(f)


def _run(exe, algo, X, Y, *extra):
    d = tempfile.mkdtemp()
    px, py = os.path.join(d, "x.bin"), os.path.join(d, "y.bin")
    _write(px, X)
    _write(py, Y)
    r = subprocess.run([exe, algo, px, py] + [str(e) for e in extra], capture_output=True, text=True)
    vals = [float(v) for v in r.stdout.split()]
    return np.array(vals[:9]).reshape(3, 3), np.array(vals[9:12]), int(vals[12]), r.stderr


def test_dropin_without_gpu_reports_and_keeps_pose(dropin_exe):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    X = np.random.default_rng(0).uniform(0, 1, (30, 3))
    R, t, ok, err = _run(dropin_exe, "emicp", X, X)
    assert np.array_equal(R, np.eye(3)) and np.array_equal(t, np.zeros(3))
    assert "no usable CUDA device" in err and ok == 1


@pytest.mark.gpu
def test_dropin_emicp_and_softassign_match_oracle(dropin_exe, oracle):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.uniform_pair(n=500, seed=31, max_deg=15.0, t_range=0.05)
    R, t, ok, err = _run(dropin_exe, "emicp", X, Y)
    Ro, to, _ = oracle.emicp(X, Y)
    assert ok == 1 and err == ""
    assert rot_err_deg(R, Ro) < 1e-3 and np.abs(t - to).max() < 1e-5
    X, Y, _, _ = W.surface_pair(n=200, seed=32)
    R, t, ok, err = _run(dropin_exe, "softassign", X, Y)
    Ro, to, _ = oracle.softassign(X, Y)
    assert rot_err_deg(R, Ro) < 1e-3


@pytest.mark.gpu
def test_dropin_icp_matches_oracle(dropin_exe, oracle):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.uniform_pair(n=800, seed=33, max_deg=15.0, t_range=0.05)
    R, t, ok, err = _run(dropin_exe, "icp", X, Y)
    Ro, to, _, _ = oracle.icp(X, Y)
    assert ok == 1 and err == ""
    assert rot_err_deg(R, Ro) < 1e-3 and np.abs(t - to).max() < 1e-5


def _identity_printout():
    return "R\n" + "".join("%f %f %f \n" % tuple(r) for r in np.eye(3)) + "t\n%f %f %f \n" % (0.0, 0.0, 0.0)


def test_dropin_emicp_cpu_and_printRT_without_gpu(dropin_exe):
    """emicp_cpu() and printRT() are declared and link; without a GPU,
    emicp_cpu reports the failure and keeps the pose, and printRT prints it in
    the reference CLI's layout (src/main.cpp:184-195)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    X = np.random.default_rng(0).uniform(0, 1, (30, 3))
    R, t, ok, err = _run(dropin_exe, "emicp_cpu", X, X)
    assert np.array_equal(R, np.eye(3)) and np.array_equal(t, np.zeros(3))
    assert "emicp_cpu: runs the GPU EM-ICP" in err and "no usable CUDA device" in err
    d = tempfile.mkdtemp()
    px = os.path.join(d, "x.bin")
    _write(px, X)
    r = subprocess.run([dropin_exe, "printRT", px, px], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout == _identity_printout()


@pytest.mark.gpu
def test_dropin_emicp_cpu_and_printRT_match_emicp(dropin_exe, oracle):
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.uniform_pair(n=500, seed=34, max_deg=15.0, t_range=0.05)
    R1, t1, ok1, err1 = _run(dropin_exe, "emicp", X, Y)
    R2, t2, ok2, err2 = _run(dropin_exe, "emicp_cpu", X, Y)
    assert ok1 == ok2 == 1 and err1 == ""
    assert "emicp_cpu: runs the GPU EM-ICP" in err2
    assert np.array_equal(R1, R2) and np.array_equal(t1, t2)
    Ro, to, _ = oracle.emicp(X, Y)
    assert rot_err_deg(R2, Ro) < 1e-3 and np.abs(t2 - to).max() < 1e-5
    d = tempfile.mkdtemp()
    px, py = os.path.join(d, "x.bin"), os.path.join(d, "y.bin")
    _write(px, X)
    _write(py, Y)
    r = subprocess.run([dropin_exe, "printRT", px, py], capture_output=True, text=True)
    lines = r.stdout.splitlines()
    assert r.returncode == 0 and lines[0] == "R" and lines[4] == "t" and len(lines) == 6
    R9 = np.array([float(v) for row in lines[1:4] for v in row.split()]).reshape(3, 3)
    tt = np.array([float(v) for v in lines[5].split()])
    assert np.abs(R9 - R1).max() <= 5e-7 and np.abs(tt - t1).max() <= 5e-7  # "%f" keeps 6 decimals
    assert all(row.endswith(" ") for row in lines[1:4] + lines[5:6])
