"""Build recipe for the oracle (test infrastructure only).

* ``oracle/libcesa_oracle.so``  -- the CPU restatement in ``cesa_oracle.c``
  (gcc + OpenMP; builds on x86_64 and aarch64).
* ``oracle/_ref/libref_emicp.so`` -- the reference's own ``emicp_cpu()`` and
  ``findRTfromS()``, compiled unmodified from the reference sources
  (src/emicp_cpu.cpp, src/findRTfromS.cpp, src/cloud2data.cpp) with the header
  stubs in ``oracle/stubs`` and ``-DNOVIEWER``.  BLAS/LAPACK come from the
  OpenBLAS that scipy bundles, through ``blas_trampoline.c``.  Built only where
  the reference tree is present (``CESA_REFERENCE_DIR``, default
  ``/root/reference``); it is never shipped and never part of the product.

Run ``python oracle/build.py`` or call :func:`build`.
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
ORACLE_SO = os.path.join(HERE, "libcesa_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libref_emicp.so")


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    srcs = [os.path.join(HERE, "cesa_oracle.c"), os.path.join(HERE, "oracle_impl.h")]
    if force or _stale(ORACLE_SO, srcs):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11",
              "-o", ORACLE_SO, srcs[0], "-lm"])
    return ORACLE_SO


def _scipy_openblas():
    try:
        import scipy
    except ImportError:
        return None
    libs = os.path.join(os.path.dirname(scipy.__file__), os.pardir, "scipy.libs")
    cands = sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so*")))
    cands = [c for c in cands if "openblas64" not in os.path.basename(c)]
    return os.path.abspath(cands[0]) if cands else None


def reference_dir():
    return os.environ.get("CESA_REFERENCE_DIR", "/root/reference")


def build_reference(force=False):
    """Compile the reference's CPU EM-ICP; returns the .so path or None."""
    src = os.path.join(reference_dir(), "src")
    needed = [os.path.join(src, f) for f in ("emicp_cpu.cpp", "findRTfromS.cpp", "cloud2data.cpp",
                                             "3dregistration.h")]
    if not all(os.path.exists(p) for p in needed):
        return None
    blas = _scipy_openblas()
    if blas is None:
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    ours = [os.path.join(HERE, "ref_entry.cpp"), os.path.join(HERE, "blas_trampoline.c")]
    if not (force or _stale(REF_SO, needed + ours)):
        return REF_SO
    tramp_o = os.path.join(REF_DIR, "blas_trampoline.o")
    _run(["gcc", "-O2", "-fPIC", "-c", ours[1], "-o", tramp_o])
    # The reference tree comes before ours, so ref_entry.cpp sees the reference's own
    # 3dregistration.h (which declares emicp_cpu); ours supplies cesa_pcl_compat.h.
    inc = ["-I", os.path.join(HERE, "stubs"), "-I", src, "-I", os.path.join(REPO, "include")]
    _run(["g++", "-O3", "-fPIC", "-shared", "-fopenmp", "-DNOVIEWER", "-w"] + inc +
         [needed[0], needed[1], needed[2], ours[0], tramp_o, "-o", REF_SO,
          blas, "-Wl,-rpath," + os.path.dirname(blas)])
    return REF_SO


def build(force=False):
    out = {"oracle": build_oracle(force)}
    try:
        out["reference"] = build_reference(force)
    except subprocess.CalledProcessError as e:  # the reference is optional
        print("reference CPU build failed:", e, file=sys.stderr)
        out["reference"] = None
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
