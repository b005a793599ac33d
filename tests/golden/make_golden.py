"""Generates the golden fixtures in this directory from the reference's own
code, built from the reference sources by oracle/build.py:

* emicp_reference.npz, findrt_reference.npz -- emicp_cpu() and findRTfromS()
  (src/emicp_cpu.cpp, src/findRTfromS.cpp, compiled unmodified into
  oracle/_ref/libref_emicp.so);
* softassign_reference.npz, emicp_gpu_reference.npz -- the reference's GPU
  softassign() and emicp() (src/softassign.cu, src/emicp.cu), their CUDA
  kernels and cuBLAS calls run on the host by oracle/emu
  (oracle/_ref/libref_gpu.so), with the reference's own per-update record of
  Xc, Yc, S, R, t (taken at its findRTfromS calls).

Run where the reference tree is available:
    python tests/golden/make_golden.py [gpu | softassign | emicp]
("gpu" makes only the last two, "softassign" / "emicp" one of them). The fixtures store the seeded inputs next to
the reference's outputs, so the tests that read them need neither the
reference tree nor the generator.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from cuda_emicp_softassign_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402


def emicp_cases():
    cases = []
    for n, seed in ((101, 11), (257, 12), (1007, 13)):
        X, Y, R, t = W.uniform_pair(n=n, seed=seed)
        cases.append(("uniform_%d" % n, X, Y))
    X, Y, R, t = W.uniform_pair(n=300, m=200, seed=14)
    cases.append(("uniform_300x200", X, Y))
    X, Y, R, t = W.surface_pair(n=400, seed=15, max_deg=20.0, outlier_frac=0.05)
    cases.append(("surface_400", X, Y))
    return cases


def softassign_cases():
    """(name, X, Y, schedule) of the reference Softassign fixtures."""
    d = dict(JMAX=100, I0=5, I1=3, alpha=3.0, T_0=100.0, TFACTOR=0.95)
    cases = []
    _, X, Y, _, _ = W.make("c2_softassign_2000", seed=0)
    cases.append(("c2_first_updates", X, Y, dict(d, JMAX=1, I0=2)))
    X, Y, _, _ = W.surface_pair(n=120, m=100, seed=3)
    for T in (100.0, 1.0, 0.05):
        cases.append(("surface_120x100_T%g" % T, X, Y, dict(d, JMAX=1, I0=1, T_0=T)))
    X, Y, _, _ = W.surface_pair(n=150, m=130, seed=4)
    cases.append(("surface_150x130_T1_50updates", X, Y, dict(d, JMAX=10, T_0=1.0)))
    X, Y, _, _ = W.surface_pair(n=100, m=100, seed=5)
    cases.append(("surface_100_default_schedule", X, Y, dict(d)))
    X, Y, _, _ = W.surface_pair(n=17, m=33, seed=6)
    cases.append(("ragged_17x33_I1_1", X, Y, dict(d, JMAX=4, I0=2, I1=1, T_0=0.5)))
    X, Y, _, _ = W.surface_pair(n=33, m=17, seed=7)
    cases.append(("ragged_33x17_I1_5", X, Y, dict(d, JMAX=4, I0=2, I1=5, T_0=0.5)))
    X, Y, _, _ = W.surface_pair(n=300, m=260, seed=9)
    cases.append(("surface_300x260_T0.1", X, Y, dict(d, JMAX=6, T_0=0.1)))
    return cases


def make_gpu_reference(parts=("softassign", "emicp")):
    """The reference's GPU softassign() and emicp() on the host (oracle/emu)."""
    if O.ref_gpu() is None:
        raise SystemExit("reference GPU-code build unavailable (needs the reference tree and scipy)")
    O.set_threads(os.cpu_count() or 1)
    if "softassign" in parts:
        make_softassign_reference()
    if "emicp" in parts:
        make_emicp_gpu_reference()


def make_softassign_reference():
    keys = ("JMAX", "I0", "I1", "alpha", "T_0", "TFACTOR")
    out = {}
    names = []
    for name, X, Y, sch in softassign_cases():
        R, t, tr = O.ref_softassign(X, Y, **sch)
        names.append(name)
        out.update({name + "_X": X, name + "_Y": Y, name + "_R": R, name + "_t": t, name + "_trace": tr,
                    name + "_sched": np.array([sch[k] for k in keys], dtype=np.float64)})
        print("softassign", name, len(tr), "updates", flush=True)
    np.savez_compressed(os.path.join(HERE, "softassign_reference.npz"), names=np.array(names), **out)


def make_emicp_gpu_reference():
    out, names = {}, []
    params = dict(sigma_p2=0.01, sigma_inf=1e-5, sigma_factor=0.9, d_02=0.01)
    for name, X, Y in emicp_cases()[2:]:
        R, t, tr = O.ref_emicp_gpu(X, Y, **params)
        names.append(name)
        out.update({name + "_X": X, name + "_Y": Y, name + "_R": R, name + "_t": t, name + "_trace": tr})
        print("emicp.cu", name, len(tr), "steps", flush=True)
    np.savez_compressed(os.path.join(HERE, "emicp_gpu_reference.npz"), names=np.array(names), **out)


def main():
    parts = [a for a in sys.argv[1:] if a in ("softassign", "emicp")]
    if "gpu" in sys.argv[1:] or parts:
        return make_gpu_reference(parts or ("softassign", "emicp"))
    if O.ref() is None:
        raise SystemExit("reference CPU build unavailable (needs the reference tree and scipy)")
    out = {}
    params = dict(sigma_p2=0.01, sigma_inf=1e-5, sigma_factor=0.9, d_02=0.01)
    for name, X, Y in emicp_cases():
        R, t = O.ref_emicp_cpu(X, Y, **params)
        out["emicp_" + name + "_X"] = X
        out["emicp_" + name + "_Y"] = Y
        out["emicp_" + name + "_R"] = R
        out["emicp_" + name + "_t"] = t
    np.savez_compressed(os.path.join(HERE, "emicp_reference.npz"), names=np.array([c[0] for c in emicp_cases()]),
                        params=np.array([params[k] for k in ("sigma_p2", "sigma_inf", "sigma_factor", "d_02")],
                                        dtype=np.float32), **out)
    rng = np.random.default_rng(2024)
    K = 64
    S = rng.standard_normal((K, 9)).astype(np.float32)
    # a few near-rotations (well separated top eigenvalue) and scaled cases
    for k in range(0, K, 4):
        A = W.random_rotation(rng, 180.0)
        S[k] = (A.reshape(-1, order="F") * rng.uniform(0.1, 10)).astype(np.float32)
    Xc = rng.standard_normal((K, 3)).astype(np.float32)
    Yc = rng.standard_normal((K, 3)).astype(np.float32)
    Rr = np.zeros((K, 3, 3))
    tr = np.zeros((K, 3))
    for k in range(K):
        Rr[k], tr[k] = O.ref_find_rt_from_s(Xc[k], Yc[k], S[k])
    np.savez_compressed(os.path.join(HERE, "findrt_reference.npz"), S=S, Xc=Xc, Yc=Yc, R=Rr, t=tr)
    make_gpu_reference()
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
