"""Generates the golden fixtures in this directory from the reference's own
CPU code (emicp_cpu() and findRTfromS(), compiled unmodified from the
reference sources by oracle/build.py into oracle/_ref/libref_emicp.so).

Run where the reference tree is available:  python tests/golden/make_golden.py
The fixtures store the seeded inputs next to the reference's outputs, so the
tests that read them need neither the reference tree nor the generator.
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


def main():
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
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
