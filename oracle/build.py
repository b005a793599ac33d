"""Build recipe for the oracle (test infrastructure only).

* ``oracle/libcesa_oracle.so``  -- the CPU restatement in ``cesa_oracle.c``
  (gcc + OpenMP; builds on x86_64 and aarch64).
* ``oracle/_ref/libref_emicp.so`` -- the reference's own ``emicp_cpu()`` and
  ``findRTfromS()``, compiled unmodified from the reference sources
  (src/emicp_cpu.cpp, src/findRTfromS.cpp, src/cloud2data.cpp and the header
  src/3dregistration.h) with the header stubs in ``oracle/stubs`` and
  ``-DNOVIEWER``.  BLAS/LAPACK come from the OpenBLAS that scipy bundles,
  through ``blas_trampoline.c``.  It is never shipped and never part of the
  product.

Where the sources come from: the reference tree (``CESA_REFERENCE_DIR``, else
the checkout this recipe was written against, ``/root/reference``). When that
tree is present the four files are also staged, unmodified, into
``oracle/_ref/src/``. ``oracle/_ref/`` is git-ignored (nothing of the
reference enters the repository's history) but travels with a copy of the
working tree, so a machine without the reference tree -- the aarch64 GPU host,
where the x86_64 build cannot run -- compiles the reference from the staged
copies.

Run ``python oracle/build.py`` or call :func:`build`.
"""
import glob
import os
import re
import shutil
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


REF_FILES = ("emicp_cpu.cpp", "findRTfromS.cpp", "cloud2data.cpp", "3dregistration.h", "softassign.cu", "emicp.cu")
REF_GPU_SO = os.path.join(REF_DIR, "libref_gpu.so")
EMU = os.path.join(HERE, "emu")
# findRTfromS(const float*, const float*, const float*, float*, float*) (src/findRTfromS.cpp:33)
FIND_RT_MANGLED = "_Z11findRTfromSPKfS0_S0_PfS1_"
STAGED_SRC = os.path.join(REF_DIR, "src")


def reference_dir():
    """The reference tree, or None where it is absent."""
    d = os.environ.get("CESA_REFERENCE_DIR", "/root/reference")
    return d if os.path.isdir(os.path.join(d, "src")) else None


def reference_sources():
    """Directory holding the reference's CPU EM-ICP sources: the reference
    tree's src/ (after staging copies into oracle/_ref/src/), else the staged
    copies, else None."""
    d = reference_dir()
    if d is not None:
        src = os.path.join(d, "src")
        if all(os.path.exists(os.path.join(src, f)) for f in REF_FILES):
            os.makedirs(STAGED_SRC, exist_ok=True)
            for f in REF_FILES:
                dst = os.path.join(STAGED_SRC, f)
                if _stale(dst, [os.path.join(src, f)]):
                    shutil.copyfile(os.path.join(src, f), dst)
            return src
    if all(os.path.exists(os.path.join(STAGED_SRC, f)) for f in REF_FILES):
        return STAGED_SRC
    return None


def build_reference(force=False):
    """Compile the reference's CPU EM-ICP; returns the .so path or None."""
    src = reference_sources()
    if src is None:
        return None
    needed = [os.path.join(src, f) for f in REF_FILES]
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


def rewrite_launches(src):
    """The reference CUDA source with every kernel launch
    `kernel <<< grid, block >>> (args);` written as
    `cesa_emu::Launch(grid, block).run([&] { kernel(args); });`, the form the
    host emulation in oracle/emu runs. Nothing else changes (line numbers
    included)."""
    out, i = [], 0
    pat = re.compile(r"(\w+)(\s*)<<<")
    while True:
        m = pat.search(src, i)
        if not m:
            out.append(src[i:])
            return "".join(out)
        cfg_end = src.index(">>>", m.end())
        cfg = src[m.end():cfg_end]
        j = cfg_end + 3
        while src[j].isspace():
            j += 1
        if src[j] != "(":
            raise ValueError("unexpected launch syntax near offset %d" % m.start())
        depth, k = 0, j
        while True:
            depth += {"(": 1, ")": -1}.get(src[k], 0)
            if depth == 0:
                break
            k += 1
        out.append(src[i:m.start()])
        out.append("cesa_emu::Launch(%s).run([&] {%s%s%s(%s); })" % (cfg, m.group(2), src[cfg_end + 3:j], m.group(1),
                                                                    src[j + 1:k]))
        i = k + 1


def build_reference_gpu(force=False):
    """The reference's own softassign() and emicp() (src/softassign.cu,
    src/emicp.cu), their CUDA kernels and cuBLAS calls run on the host by
    oracle/emu; returns the .so path or None. The link wraps findRTfromS so
    that every pose update is recorded."""
    src = reference_sources()
    if src is None:
        return None
    blas = _scipy_openblas()
    if blas is None:
        return None
    needed = [os.path.join(src, f) for f in ("softassign.cu", "emicp.cu", "findRTfromS.cpp", "cloud2data.cpp",
                                             "3dregistration.h")]
    ours = [os.path.join(HERE, "ref_gpu_entry.cpp"), os.path.join(HERE, "blas_trampoline.c")] + \
        [os.path.join(EMU, f) for f in ("cuda_emu.h", "cublas.h", "helper_cuda.h", "helper_timer.h",
                                        "emu_runtime.cpp")]
    if not (force or _stale(REF_GPU_SO, needed + ours + [__file__])):
        return REF_GPU_SO
    os.makedirs(REF_DIR, exist_ok=True)
    gens = []
    for cu in needed[:2]:
        gen = os.path.join(REF_DIR, os.path.splitext(os.path.basename(cu))[0] + "_emu.cpp")
        with open(cu) as f:
            text = rewrite_launches(f.read())
        with open(gen, "w") as f:
            f.write("// Generated by oracle/build.py from the reference's src/%s: kernel launches rewritten for\n"
                    "// the host emulation in oracle/emu; not part of the repository.\n" % os.path.basename(cu))
            f.write(text)
        gens.append(gen)
    inc = ["-I", EMU, "-I", os.path.join(HERE, "stubs"), "-I", src, "-I", os.path.join(REPO, "include")]
    cxx = ["g++", "-O2", "-fPIC", "-fopenmp", "-DNOVIEWER", "-w", "-std=c++17"]
    objs = []
    for name, extra in ((gens[0], ["-include", "cuda_emu.h"]), (gens[1], ["-include", "cuda_emu.h"]),
                        (needed[2], []), (needed[3], []), (os.path.join(EMU, "emu_runtime.cpp"), []),
                        (ours[0], ["-DCESA_FIND_RT_WRAP=__wrap_" + FIND_RT_MANGLED,
                                   "-DCESA_FIND_RT_REAL=__real_" + FIND_RT_MANGLED])):
        o = os.path.join(REF_DIR, "sa_" + os.path.splitext(os.path.basename(name))[0] + ".o")
        _run(cxx + extra + inc + ["-c", name, "-o", o])
        objs.append(o)
    tramp_o = os.path.join(REF_DIR, "blas_trampoline.o")
    _run(["gcc", "-O2", "-fPIC", "-c", ours[1], "-o", tramp_o])
    _run(["g++", "-shared", "-fopenmp", "-o", REF_GPU_SO] + objs + [tramp_o, "-Wl,--wrap=" + FIND_RT_MANGLED, blas,
                                                                    "-Wl,-rpath," + os.path.dirname(blas)])
    return REF_GPU_SO


def build(force=False):
    out = {"oracle": build_oracle(force)}
    try:
        out["reference"] = build_reference(force)
    except subprocess.CalledProcessError as e:  # the reference is optional
        print("reference CPU build failed:", e, file=sys.stderr)
        out["reference"] = None
    try:
        out["reference_gpu"] = build_reference_gpu(force)
    except (subprocess.CalledProcessError, ValueError) as e:
        print("reference GPU code (host emulation) build failed:", e, file=sys.stderr)
        out["reference_gpu"] = None
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
