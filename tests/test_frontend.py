"""Point-cloud front end and command line (cesa_load_points, cesa_points_reduction,
cesa_align_scale_once, cesa_save_rt / cesa_load_rt, cesa_register): the
reference CLI's loadFile, pointsReduction, alignScaleOnce, saveRTtoFile,
loadRTfromFile and main (src/main.cpp:41-499), headless and without PCL.

CPU tests write PLY / text files in every layout the loader accepts and read
them back; the GPU tests run cesa_register end to end against the oracle.
"""
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import rot_err_deg


def _pts(n=50, seed=0):
    return np.random.default_rng(seed).uniform(-1, 1, (n, 3)).astype(np.float32)


def _write_ply_ascii(path, P, extra_before=False, faces=True):
    with open(path, "w") as f:
        f.write("ply\nformat ascii 1.0\ncomment made by a test\nobj_info num_cols 3\n")
        if extra_before:
            f.write("element camera 1\nproperty float view_px\nproperty float view_py\n")
        f.write("element vertex %d\nproperty float x\nproperty float y\nproperty float z\n" % len(P))
        f.write("property float confidence\nproperty uchar red\n")
        if faces:
            f.write("element face 1\nproperty list uchar int vertex_indices\n")
        f.write("end_header\n")
        if extra_before:
            f.write("0.5 0.25\n")
        for p in P:
            f.write("%.9g %.9g %.9g 0.9 255\n" % tuple(p))
        if faces:
            f.write("3 0 1 2\n")


def _write_ply_binary(path, P, big=False, double=False):
    fmt = "binary_big_endian" if big else "binary_little_endian"
    typ = "double" if double else "float"
    e = ">" if big else "<"
    c = "d" if double else "f"
    with open(path, "wb") as f:
        f.write(("ply\nformat %s 1.0\nelement vertex %d\nproperty uchar flags\nproperty %s x\n"
                 "property %s y\nproperty %s z\nproperty short s\nelement face 1\n"
                 "property list uchar int vertex_indices\nend_header\n" % (fmt, len(P), typ, typ, typ)).encode())
        for p in P:
            f.write(struct.pack(e + "B" + c * 3 + "h", 7, float(p[0]), float(p[1]), float(p[2]), -3))
        f.write(struct.pack(e + "Biii", 3, 0, 1, 2))


@pytest.mark.parametrize("layout", ["ascii", "ascii_extra", "le_float", "be_float", "le_double", "be_double"])
def test_ply_layouts(cesa, layout):
    P = _pts()
    d = tempfile.mkdtemp()
    path = os.path.join(d, "c.ply")
    if layout.startswith("ascii"):
        _write_ply_ascii(path, P, extra_before=layout == "ascii_extra")
    else:
        _write_ply_binary(path, P, big=layout.startswith("be"), double=layout.endswith("double"))
    Q = cesa.load_points(path)
    assert Q.shape == P.shape and np.array_equal(Q, P)


def test_text_and_non_finite_points(cesa):
    P = _pts(20, 1)
    d = tempfile.mkdtemp()
    path = os.path.join(d, "c.txt")
    with open(path, "w") as f:
        f.write("# x y z\n\n")
        for i, p in enumerate(P):
            if i == 5:
                f.write("nan 0 0\n")
            if i == 9:
                f.write("1 inf 2 7\n")
            f.write("%.9g %.9g %.9g 1.0\n" % tuple(p))
    Q = cesa.load_points(path)
    assert np.array_equal(Q, P)  # the two non-finite points are dropped, the rest keep their order
    ply = os.path.join(d, "n.ply")
    R = P.copy()
    R[3, 1] = np.nan
    _write_ply_binary(ply, R)
    assert np.array_equal(cesa.load_points(ply), np.delete(P, 3, axis=0))


def test_bad_files_are_rejected(cesa):
    d = tempfile.mkdtemp()
    for name, body in (("a.ply", b"ply\nformat ascii 1.0\nelement vertex 2\nproperty float x\nend_header\n1\n2\n"),
                       ("b.ply", b"ply\nformat ascii 1.0\nelement vertex 3\nproperty float x\nproperty float y\n"
                                 b"property float z\nend_header\n1 2 3\n"),
                       ("c.txt", b"1 2\n")):
        path = os.path.join(d, name)
        with open(path, "wb") as f:
            f.write(body)
        with pytest.raises(cesa.CesaError):
            cesa.load_points(path)
    with pytest.raises(cesa.CesaError):
        cesa.load_points(os.path.join(d, "missing.ply"))


def test_reference_bunny_scan_loads():
    """The reference's own scan data, where the reference tree is present."""
    from oracle import build as ob
    ref = ob.reference_dir()
    path = os.path.join(ref, "data", "bun000.ply") if ref else ""
    if not path or not os.path.exists(path):
        pytest.skip("reference data not present")
    import cuda_emicp_softassign_gb300 as cesa
    n = 0
    first = None
    with open(path) as f:
        for line in f:
            w = line.split()
            if w[:2] == ["element", "vertex"]:
                n = int(w[2])
            if w == ["end_header"]:
                first = np.array(next(f).split()[:3], dtype=np.float32)
                break
    P = cesa.load_points(path)
    assert len(P) <= n and len(P) > 0.9 * n
    assert np.array_equal(P[0], first)


def test_points_reduction(cesa):
    P = _pts(20000, 2)
    a = cesa.points_reduction(P, 5.0, seed=7)
    b = cesa.points_reduction(P, 5.0, seed=7)
    c = cesa.points_reduction(P, 5.0, seed=8)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert abs(len(a) / len(P) - 0.05) < 0.006
    # kept points are a subsequence of the input, in order
    idx = [int(np.flatnonzero((P == q).all(1))[0]) for q in a[:50]]
    assert idx == sorted(idx)
    assert len(cesa.points_reduction(P, 100.0)) == len(P) and len(cesa.points_reduction(P, 0.0)) == 0


def test_align_scale_once(cesa):
    X = _pts(3000, 3) * 7.0 + 2.0
    Y = _pts(2000, 4) * 0.01 - 1.0
    A, B = cesa.align_scale_once(X, Y)
    for P, Q in ((X, A), (Y, B)):
        tr = np.trace(np.cov(Q.astype(np.float64).T, bias=True))
        assert abs(tr - 0.003) < 1e-6
        s = float(np.linalg.norm(Q) / np.linalg.norm(P))  # a scale about the origin
        assert np.allclose(Q, P * s, rtol=1e-5, atol=1e-7)


def test_rt_file_format(cesa):
    d = tempfile.mkdtemp()
    path = os.path.join(d, "rt.txt")
    R = np.array([[0.5, -0.25, 0.125], [1.0, 2.0, 3.0], [-1.5, 0.0, 1e-3]])
    t = np.array([0.1, -0.2, 0.3])
    cesa.save_rt(path, R, t)
    ref = "".join("%f " % v + ("\n" if (i + 1) % 3 == 0 else "") for i, v in enumerate(R.reshape(-1).astype(np.float32)))
    ref += "".join("%f " % v for v in t.astype(np.float32)) + "\n"
    assert open(path).read() == ref
    R2, t2 = cesa.load_rt(path)
    assert np.allclose(R2, R, atol=1e-6) and np.allclose(t2, t, atol=1e-6)


def _cli(cesa, *args):
    from cuda_emicp_softassign_gb300 import build
    exe = build.build_cli()
    return subprocess.run([exe] + list(args), capture_output=True, text=True)


def _write_pair(d, X, Y):
    px, py = os.path.join(d, "x.ply"), os.path.join(d, "y.txt")
    _write_ply_binary(px, X)
    with open(py, "w") as f:
        for p in Y:
            f.write("%.9g %.9g %.9g\n" % tuple(p))
    return px, py


def test_cli_arguments_and_front_end_without_gpu(cesa):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = _cli(cesa)
    assert r.returncode == 1 and "pointFileX" in r.stderr
    d = tempfile.mkdtemp()
    px, py = _write_pair(d, _pts(400, 5), _pts(300, 6))
    out = os.path.join(d, "rt.txt")
    r = _cli(cesa, "-pointFileX=" + px, "-pointFileY=" + py, "-emicp", "-noviewer", "-pointsReductionRate=50",
             "-seed=3", "-saveRTtoFile=" + out)
    assert r.returncode == 1 and "no usable CUDA device" in r.stderr
    assert "EM-ICP paramters" in r.stdout and "sigma_p2 0.01" in r.stdout
    sizes = [int(l.split()[1]) for l in r.stdout.splitlines() if l.startswith(("Xsize", "Ysize"))]
    assert 150 < sizes[0] < 250 and 100 < sizes[1] < 200
    R, t = cesa.load_rt(out)
    assert np.array_equal(R, np.eye(3)) and np.array_equal(t, np.zeros(3))


@pytest.mark.gpu
@pytest.mark.parametrize("algo", ["emicp", "icp", "softassign"])
def test_cli_registers_like_the_oracle(cesa, oracle, algo):
    from cuda_emicp_softassign_gb300 import workloads as W
    if algo == "softassign":
        X, Y, _, _ = W.surface_pair(n=300, seed=12)
    else:
        X, Y, _, _ = W.uniform_pair(n=700, seed=11, max_deg=15.0, t_range=0.05)
    d = tempfile.mkdtemp()
    px, py = _write_pair(d, X, Y)
    rt0, rt1 = os.path.join(d, "rt0.txt"), os.path.join(d, "rt1.txt")
    cesa.save_rt(rt0, np.eye(3), np.zeros(3))
    args = ["-pointFileX=" + px, "-pointFileY=" + py, "-noviewer", "-loadRTfromFile=" + rt0, "-saveRTtoFile=" + rt1]
    if algo != "softassign":
        args.append("-" + algo)
    r = _cli(cesa, *args)
    assert r.returncode == 0, r.stderr
    assert "elapsed" in r.stdout
    R, t = cesa.load_rt(rt1)
    if algo == "emicp":
        Ro, to, _ = oracle.emicp(X, Y)
    elif algo == "icp":
        Ro, to, _, _ = oracle.icp(X, Y)
    else:
        Ro, to, _ = oracle.softassign(X, Y)
    # the file holds %f (6 decimals)
    assert rot_err_deg(R, Ro) < 2e-3 and np.abs(t - to).max() < 2e-6 + 1e-5
