"""Builds libcesa.so (the C ABI declared in include/cesa.h) for sm_103a.

Each ``csrc/*.cu`` file is compiled in parallel with nvcc, then linked into
``cuda_emicp_softassign_gb300/libcesa.so`` with a static CUDA runtime. A
version script exports only the ``cesa_*`` symbols. Object files go to
``cuda_emicp_softassign_gb300/_build/``.

Run ``python -m cuda_emicp_softassign_gb300.build`` or call :func:`build`.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcesa.so")
PEAKS_LIB = os.path.join(HERE, "libcesa_peaks.so")
CLI = os.path.join(HERE, "cesa_register")
TOOLS = os.path.join(HERE, "cesa_tools")
TOOL_NAMES = ("add_rigid_transform", "merge", "pcd2ply")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no contraction into fused multiply-adds, so that it rounds the
# same on x86_64 and aarch64 (gcc contracts by default on aarch64)
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE]
SOURCES = ["cesa_api.cu", "cesa_emicp.cu", "cesa_softassign.cu", "cesa_noalloc.cu", "cesa_selftest.cu",
           "cesa_batch.cu", "cesa_softassign_mat.cu", "cesa_emicp_adjoint.cu",
           "cesa_softassign_adjoint.cu", "cesa_icp.cu", "cesa_io.cpp", "cesa_softassign_band.cu"]
HEADERS = ["cesa_common.cuh", "cesa_sweep.cuh", "cesa_pose.h", "cesa_kernels.h", "cesa_prep.cuh", "cesa_ops.cuh",
           "cesa_sa_pose.cuh"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcesa.so")


def _mtime(p):
    return os.path.getmtime(p) if os.path.exists(p) else 0.0


def _deps_mtime():
    paths = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "cesa.h"), __file__]
    return max(_mtime(p) for p in paths)


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    s = os.path.join(CSRC, src)
    if _mtime(obj) >= max(_mtime(s), _deps_mtime()):
        return obj
    cmd = [nvcc()] + NVFLAGS + ["-c", s, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force=False, verbose=False):
    """Compiles and links libcesa.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if _mtime(LIB) >= max(_mtime(o) for o in objs) and not force:
        return LIB
    vs = os.path.join(BUILD, "exports.map")
    with open(vs, "w") as f:
        f.write("{ global: cesa_*; local: *; };\n")
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + [
        "-Xlinker", "--version-script=" + vs, "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


def _build_exe(src_name, out, force):
    """Compiles one host C++ executable over libcesa.so (found beside it)."""
    lib = build()
    src = os.path.join(CSRC, src_name)
    if not force and _mtime(out) >= max(_mtime(src), _mtime(lib), _mtime(os.path.join(INCLUDE, "cesa.h"))):
        return out
    tmp = out + ".tmp"
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", INCLUDE, src, "-L", HERE, "-lcesa",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed for %s:\n%s\n%s" % (src_name, r.stdout, r.stderr))
    os.replace(tmp, out)
    return out


def build_cli(force=False):
    """Compiles the cesa_register command line; returns its path."""
    return _build_exe("cesa_cli.cpp", CLI, force)


def build_tools(force=False):
    """Compiles the point-cloud tools (one executable, cesa_tools) and links
    the names it answers to beside it; returns {tool name: path}."""
    exe = _build_exe("cesa_tools.cpp", TOOLS, force)
    out = {}
    for name in TOOL_NAMES:
        path = os.path.join(HERE, name)
        if os.path.islink(path) or os.path.exists(path):
            if os.path.islink(path) and os.readlink(path) == os.path.basename(exe):
                out[name] = path
                continue
            os.remove(path)
        os.symlink(os.path.basename(exe), path)
        out[name] = path
    return out


def build_peaks(force=False):
    """Compiles libcesa_peaks.so (FP32 / MUFU throughput probes for bench.py)."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(CSRC, "cesa_peaks.cu")
    if not force and _mtime(PEAKS_LIB) >= _mtime(src):
        return PEAKS_LIB
    tmp = PEAKS_LIB + ".tmp"
    cmd = [nvcc()] + NVFLAGS + ["-shared", src, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for cesa_peaks.cu:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, PEAKS_LIB)
    return PEAKS_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_cli(force="--force" in sys.argv))
    print(build_tools(force="--force" in sys.argv))
    print(build_peaks(force="--force" in sys.argv))
