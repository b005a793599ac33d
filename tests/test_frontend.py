"""Point-cloud front end, command line and tools (cesa_load_points,
cesa_points_reduction, cesa_align_scale_once, cesa_save_rt / cesa_load_rt,
cesa_save_points, cesa_transform_points, cesa_register, cesa_tools): the
reference CLI's loadFile, pointsReduction, alignScaleOnce, saveRTtoFile,
loadRTfromFile and main (src/main.cpp:41-499) and its point-cloud tools
(src/add_rigid_transform.cpp, src/merge.cpp, src/pcd2ply.cpp), headless and
without PCL.

CPU tests write PLY / PCD / text files in every layout the loader accepts and
read them back, and run the tools; the GPU tests run cesa_register end to end
against the oracle.
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


# ---- PCD ---------------------------------------------------------------------

def _lzf(data):
    """A small LZF encoder (literal runs of up to 32 bytes, back references of
    3 to 264 bytes within 8192), so that the loader's decoder sees both kinds
    of token, overlapping references included."""
    out, lit, last = bytearray(), bytearray(), {}
    n, i = len(data), 0

    def flush():
        for k in range(0, len(lit), 32):
            chunk = lit[k:k + 32]
            out.append(len(chunk) - 1)
            out.extend(chunk)
        lit.clear()

    while i < n:
        key = bytes(data[i:i + 3])
        j = last.get(key) if len(key) == 3 else None
        if len(key) == 3:
            last[key] = i
        if j is not None and i - j - 1 < 8192:
            L = 3
            while i + L < n and L < 264 and data[j + L] == data[i + L]:
                L += 1
            flush()
            off, e = i - j - 1, L - 2
            if e < 7:
                out.append((e << 5) | (off >> 8))
            else:
                out.append((7 << 5) | (off >> 8))
                out.append(e - 7)
            out.append(off & 255)
            i += L
        else:
            lit.append(data[i])
            i += 1
    flush()
    return bytes(out)


# a cloud with fields around x, y, z: a float "rgb" before, a padding field and
# a 3-count "normal" after (the x, y, z offsets are not at the record start)
_PCD_FIELDS = [("rgb", 4, "F", 1), ("x", 4, "F", 1), ("y", 4, "F", 1), ("z", 4, "F", 1),
               ("_", 1, "U", 4), ("normal", 8, "F", 3), ("label", 2, "U", 1)]


def _pcd_header(n, data, fields=_PCD_FIELDS, version="0.7"):
    return ("# .PCD v%s - written by a test\nVERSION %s\nFIELDS %s\nSIZE %s\nTYPE %s\nCOUNT %s\n"
            "WIDTH %d\nHEIGHT 1\nVIEWPOINT 0 0 0 1 0 0 0\nPOINTS %d\nDATA %s\n" % (
                version, version, " ".join(f[0] for f in fields), " ".join(str(f[1]) for f in fields),
                " ".join(f[2] for f in fields), " ".join(str(f[3]) for f in fields), n, n, data)).encode()


def _pcd_columns(P):
    n = len(P)
    rng = np.random.default_rng(9)
    return {"rgb": rng.uniform(0, 1, (n, 1)).astype("<f4"), "x": P[:, :1].astype("<f4"),
            "y": P[:, 1:2].astype("<f4"), "z": P[:, 2:3].astype("<f4"),
            "_": np.zeros((n, 4), "<u1"), "normal": rng.normal(size=(n, 3)).astype("<f8"),
            "label": (np.arange(n) % 7).reshape(n, 1).astype("<u2")}


def _write_pcd(path, P, data):
    cols = _pcd_columns(P)
    n = len(P)
    with open(path, "wb") as f:
        f.write(_pcd_header(n, data))
        if data == "ascii":
            for i in range(n):
                f.write((" ".join(" ".join(repr(float(v)) for v in cols[name][i])
                                  for name, _, _, _ in _PCD_FIELDS) + "\n").encode())
        elif data == "binary":
            for i in range(n):
                f.write(b"".join(cols[name][i].tobytes() for name, _, _, _ in _PCD_FIELDS))
        else:  # field-major, LZF-compressed
            raw = b"".join(cols[name].tobytes() for name, _, _, _ in _PCD_FIELDS)
            comp = _lzf(raw)
            f.write(struct.pack("<II", len(comp), len(raw)))
            f.write(comp)


@pytest.mark.parametrize("data", ["ascii", "binary", "binary_compressed"])
def test_pcd_layouts(cesa, data):
    # coordinates on a coarse lattice, so that the compressed stream holds
    # back references as well as literals
    P = (np.random.default_rng(3).integers(-20, 20, (700, 3)) / 8.0).astype(np.float32)
    P[5] = [0.1, -0.2, 0.3]
    d = tempfile.mkdtemp()
    path = os.path.join(d, "c.pcd")
    _write_pcd(path, P, data)
    Q = cesa.load_points(path)
    assert np.array_equal(Q, P)
    # detected by content as well as by name
    other = os.path.join(d, "c.cloud")
    os.replace(path, other)
    assert np.array_equal(cesa.load_points(other), P)


def test_pcd_non_finite_points_and_bad_files(cesa):
    P = _pts(30, 4)
    P[7, 2] = np.nan
    d = tempfile.mkdtemp()
    path = os.path.join(d, "n.pcd")
    _write_pcd(path, P, "binary_compressed")
    assert np.array_equal(cesa.load_points(path), np.delete(P, 7, axis=0))
    bad = {
        "nofield.pcd": _pcd_header(1, "ascii", [("x", 4, "F", 1), ("y", 4, "F", 1)]) + b"1 2\n",
        "short.pcd": _pcd_header(3, "ascii", [("x", 4, "F", 1), ("y", 4, "F", 1), ("z", 4, "F", 1)]) + b"1 2 3\n",
        "badtype.pcd": _pcd_header(1, "ascii", [("x", 3, "F", 1), ("y", 4, "F", 1), ("z", 4, "F", 1)]) + b"1 2 3\n",
        "trunc.pcd": _pcd_header(2, "binary", [("x", 4, "F", 1), ("y", 4, "F", 1), ("z", 4, "F", 1)]) + b"\0" * 20,
        # a back reference before the start of the output
        "lzf.pcd": _pcd_header(1, "binary_compressed", [("x", 4, "F", 1), ("y", 4, "F", 1), ("z", 4, "F", 1)])
        + struct.pack("<II", 2, 12) + bytes([0x20, 0x05]),
    }
    for name, body in bad.items():
        p = os.path.join(d, name)
        with open(p, "wb") as f:
            f.write(body)
        with pytest.raises(cesa.CesaError):
            cesa.load_points(p)


def _round8(a):
    """What 8 significant digits (PCL's writers) read back as FP32."""
    return np.array([float("%.8g" % float(v)) for v in np.asarray(a, np.float32).reshape(-1)],
                    np.float64).astype(np.float32).reshape(np.shape(a))


def test_save_points_formats(cesa):
    P = _pts(40, 8) * np.float32(123.456)
    P[3] = [1e-30, -3e20, 0.0]
    d = tempfile.mkdtemp()
    pcd, ply, txt = (os.path.join(d, "p." + e) for e in ("pcd", "ply", "xyz"))
    cesa.save_points(pcd, P)
    cesa.save_points(ply, P)
    cesa.save_points(txt, P)
    lines = open(pcd).read().split("\n")
    assert lines[:11] == ["# .PCD v0.7 - Point Cloud Data file format", "VERSION 0.7", "FIELDS x y z",
                          "SIZE 4 4 4", "TYPE F F F", "COUNT 1 1 1", "WIDTH 40", "HEIGHT 1",
                          "VIEWPOINT 0 0 0 1 0 0 0", "POINTS 40", "DATA ascii"]
    assert lines[11] == " ".join("%.8g" % float(v) for v in P[0])
    assert np.array_equal(cesa.load_points(pcd), _round8(P))
    assert open(ply).read().startswith("ply\nformat ascii 1.0\nelement vertex 40\n")
    assert np.array_equal(cesa.load_points(ply), _round8(P))
    assert np.array_equal(cesa.load_points(txt), P)  # 9 digits: exact
    # an explicit format wins over the name
    cesa.save_points(txt, P, cesa.POINTS_PCD)
    assert open(txt).read().startswith("# .PCD v0.7")
    cesa.save_points(pcd, np.zeros((0, 3), np.float32))
    assert cesa.load_points(pcd).shape == (0, 3)
    with pytest.raises(cesa.CesaError):
        cesa.save_points(pcd, P, 9)


def _transform_fp32(P, R, t):
    """R p + t with every product and sum rounded in FP32, left to right."""
    P = np.asarray(P, np.float32)
    R = np.asarray(R, np.float32)
    t = np.asarray(t, np.float32)
    out = np.empty_like(P)
    for r in range(3):
        out[:, r] = ((R[r, 0] * P[:, 0] + R[r, 1] * P[:, 1]) + R[r, 2] * P[:, 2]) + t[r]
    return out


def test_transform_points_rounds_like_fp32(cesa):
    from cuda_emicp_softassign_gb300 import workloads as W
    P = _pts(5000, 9) * np.float32(3.0)
    R = W.random_rotation(np.random.default_rng(2), 40.0).astype(np.float32)
    t = np.array([0.25, -1.5, 3.0], np.float32)
    assert np.array_equal(cesa.transform_points(P, R, t), _transform_fp32(P, R, t))


def _tool(name, *args):
    from cuda_emicp_softassign_gb300 import build
    exe = build.build_tools()[name]
    return subprocess.run([exe] + list(args), capture_output=True, text=True)


def test_tools_transform_merge_convert(cesa):
    from cuda_emicp_softassign_gb300 import workloads as W
    d = tempfile.mkdtemp()
    A, B = _pts(300, 10), _pts(200, 11)
    pa, pb = os.path.join(d, "a.ply"), os.path.join(d, "b.pcd")
    _write_ply_binary(pa, A)
    _write_pcd(pb, B, "binary_compressed")
    R = W.random_rotation(np.random.default_rng(5), 30.0)
    t = np.array([0.1, 0.2, -0.3])
    rt = os.path.join(d, "rt.txt")
    cesa.save_rt(rt, R, t)
    R32, t32 = cesa.load_rt(rt)

    out = os.path.join(d, "a_trans.pcd")
    r = _tool("add_rigid_transform", pa, out, rt)
    assert r.returncode == 0, r.stderr
    assert open(out).read().startswith("# .PCD v0.7")
    A2 = _round8(_transform_fp32(A, R32, t32))
    assert np.array_equal(cesa.load_points(out), A2)

    out_ply = os.path.join(d, "a_trans.ply")  # the *_ply variant the demos use
    assert _tool("add_rigid_transform", pa, out_ply, rt).returncode == 0
    assert open(out_ply).read().startswith("ply\n") and np.array_equal(cesa.load_points(out_ply), A2)

    merged = os.path.join(d, "m.pcd")
    r = _tool("merge", out, pb, merged)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(cesa.load_points(merged), np.concatenate([A2, _round8(B)]))

    conv = os.path.join(d, "m_out")  # no extension: pcd2ply writes PLY whatever the name
    r = _tool("pcd2ply", merged, conv)
    assert r.returncode == 0, r.stderr
    assert open(conv).read().startswith("ply\n")
    assert np.array_equal(cesa.load_points(conv), np.concatenate([A2, _round8(B)]))

    # the executable also takes the tool's name as its first argument
    from cuda_emicp_softassign_gb300 import build
    r = subprocess.run([build.TOOLS, "merge", pa, pa, merged], capture_output=True, text=True)
    assert r.returncode == 0 and len(cesa.load_points(merged)) == 600


def test_tools_reject_bad_arguments(cesa):
    d = tempfile.mkdtemp()
    pa = os.path.join(d, "a.ply")
    _write_ply_binary(pa, _pts(10, 12))
    for args in (("add_rigid_transform", pa, os.path.join(d, "o.pcd")),
                 ("add_rigid_transform", pa, os.path.join(d, "o.pcd"), os.path.join(d, "missing_rt.txt")),
                 ("merge", pa, os.path.join(d, "missing.ply"), os.path.join(d, "o.pcd")),
                 ("pcd2ply", os.path.join(d, "missing.pcd"), os.path.join(d, "o.ply")),
                 ("pcd2ply", pa, os.path.join(d, "no_such_dir", "o.ply"))):
        r = _tool(*args)
        assert r.returncode == 1, args
    from cuda_emicp_softassign_gb300 import build
    assert subprocess.run([build.TOOLS, "frobnicate"], capture_output=True).returncode == 1


def test_reference_bunny_demo_chain(cesa):
    """One of the reference's bunny-building demo steps (Makefile.demo:108-111)
    on its own scans, where the reference tree is present: transform bun045 by
    an RT file, merge it with bun000, convert the result to PLY."""
    from oracle import build as ob
    ref = ob.reference_dir()
    s0 = os.path.join(ref, "data", "bun000.ply") if ref else ""
    s1 = os.path.join(ref, "data", "bun045.ply") if ref else ""
    if not (s0 and os.path.exists(s0) and os.path.exists(s1)):
        pytest.skip("reference data not present")
    d = tempfile.mkdtemp()
    rt = os.path.join(d, "rt.txt")
    c, s = np.cos(np.radians(45.0)), np.sin(np.radians(45.0))
    cesa.save_rt(rt, np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]]), np.array([0.001, -0.002, 0.0005]))
    R32, t32 = cesa.load_rt(rt)
    trans, merged, conv = (os.path.join(d, f) for f in ("bun045_trans.ply", "bun1.pcd", "bun1.ply"))
    assert _tool("add_rigid_transform", s1, trans, rt).returncode == 0
    assert _tool("merge", s0, trans, merged).returncode == 0
    assert _tool("pcd2ply", merged, conv).returncode == 0
    A, B = cesa.load_points(s0), cesa.load_points(s1)
    want = np.concatenate([_round8(A), _round8(_transform_fp32(B, R32, t32))])
    assert np.array_equal(cesa.load_points(conv), want)
