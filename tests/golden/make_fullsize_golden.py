"""Generates the full-size parity fixtures of the benchmark configs.

    python tests/golden/make_fullsize_golden.py [c3] [c5] [c4] [c2] [--no-reference]

Each fixture holds the FP64 oracle's result (oracle/cesa_oracle.c, a line-cited
restatement of src/emicp_cpu.cpp:303-528 and src/softassign.cu:486-822) on the
seeded synthetic pair of a config, next to the inputs themselves, so that the
GPU tests and bench.py compare against exactly the points the oracle saw:

* c3_emicp_40097.npz -- config 3 (N = M = 40,097, 5% outliers, angle <= 20
  degrees), the whole 66-step EM-ICP schedule: the per-step trace (sum lambda,
  Xc, Yc, S, R, t) and the final pose. Also the oracle's FP32 port and, where
  the reference tree is present, the reference's own emicp_cpu() on the same
  pair (6.4 GB for its dense A matrix; about 10 minutes on 8 cores).
* c5_softassign_20000_jmax2.npz -- config 5 (N = M = 20,000) with the schedule
  cut to JMAX = 2 (10 pose updates, I0 = 5, I1 = 3): per-update trace and pose.
* c2_softassign_2000.npz -- config 2 (N = M = 2000), the whole default
  500-update schedule: per-update trace and pose (the trajectory the device
  pose solver is checked along).
* c4_emicp_pairs.npz -- the 128 EM-ICP pairs of config 4 (256 pairs, N and M
  log-uniform in [500, 20000]; the even indices of workloads.batch_pairs(256,
  seed 0)). These store no points: each pair's SHA-256 over its float32 X and Y
  bytes, so the test can check that the generator reproduced them, the
  oracle's pose, the oracle's FP32 port's pose and (where the reference tree
  is present) the reference's own emicp_cpu() pose, and `spread`: the largest
  rotation (degrees) and translation (x extent) deviation from the FP64 pose
  over C4_ENSEMBLE runs of the FP32 port on X perturbed by one ulp per
  coordinate (seeded; the FP64 pose itself moves by under 2e-6 degrees under
  such perturbations, and the port lands where it does unperturbed: its
  deviation is a bias of its evaluation order). On about 40% of these pairs
  FP32 computations of the same algorithm land apart (up to 175 degrees). As sigma^2 shrinks towards 1e-5 the weight exp(-d^2 / sigma^2)
  multiplies the FP32 rounding of d^2 (about 1e-7 on unit-cube coordinates) by
  d^2 / sigma^2, 10^2 to 10^3, so each FP32 evaluation order drifts from the
  FP64 trajectory its own way, step after step (pair 250: 1e-5 degrees after
  the first step, 3e-4 at sigma^2 = 8e-4, 0.7 at the end).
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from cuda_emicp_softassign_gb300 import workloads as W  # noqa: E402
from oracle import oracle as O  # noqa: E402

EMICP = dict(sigma_p2=0.01, sigma_inf=1e-5, sigma_factor=0.9, d_02=0.01)
C4_ENSEMBLE = 4  # perturbed FP32 runs per config-4 pair
C5_SCHED = dict(JMAX=2, I0=5, I1=3, alpha=3.0, T_0=100.0, TFACTOR=0.95)


def pair_sha(X, Y):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(X, dtype=np.float32).tobytes())
    h.update(np.ascontiguousarray(Y, dtype=np.float32).tobytes())
    return h.hexdigest()


def make_c3(with_reference):
    _, X, Y, Rt, tt = W.make("c3_emicp_40097", seed=0)
    t0 = time.time()
    R, t, tr = O.emicp(X, Y, **EMICP)
    print("c3 oracle f64: %d steps, %.0f s" % (len(tr), time.time() - t0), flush=True)
    Rp, tp, _ = O.emicp(X, Y, precision="f32", trace=False, **EMICP)
    out = dict(X=X, Y=Y, R=R, t=t, trace=tr, port_R=Rp, port_t=tp, R_true=Rt, t_true=tt,
               params=np.array([EMICP[k] for k in ("sigma_p2", "sigma_inf", "sigma_factor", "d_02")],
                               dtype=np.float32), sha=np.array(pair_sha(X, Y)))
    if with_reference and O.ref() is not None:
        t0 = time.time()
        Rr, trr = O.ref_emicp_cpu(X, Y, **EMICP)
        print("c3 reference emicp_cpu: %.0f s" % (time.time() - t0), flush=True)
        out.update(ref_R=Rr, ref_t=trr)
    np.savez_compressed(os.path.join(HERE, "c3_emicp_40097.npz"), **out)


def make_c5():
    _, X, Y, Rt, tt = W.make("c5_softassign_20000", seed=0)
    t0 = time.time()
    R, t, tr = O.softassign(X, Y, **C5_SCHED)
    print("c5 oracle f64: %d updates, %.0f s" % (len(tr), time.time() - t0), flush=True)
    Rp, tp, trp = O.softassign(X, Y, precision="f32", **C5_SCHED)
    np.savez_compressed(os.path.join(HERE, "c5_softassign_20000_jmax2.npz"), X=X, Y=Y, R=R, t=t, trace=tr,
                        port_R=Rp, port_t=tp, port_trace=trp,
                        sched=np.array([C5_SCHED[k] for k in ("JMAX", "I0", "I1", "alpha", "T_0", "TFACTOR")],
                                       dtype=np.float64), sha=np.array(pair_sha(X, Y)))


def make_c2():
    _, X, Y, Rt, tt = W.make("c2_softassign_2000", seed=0)
    t0 = time.time()
    R, t, tr = O.softassign(X, Y)
    print("c2 oracle f64: %d updates, %.0f s" % (len(tr), time.time() - t0), flush=True)
    np.savez_compressed(os.path.join(HERE, "c2_softassign_2000.npz"), X=X, Y=Y, R=R, t=t, trace=tr,
                        sha=np.array(pair_sha(X, Y)))


def fp32_spread(X, Y, R, t, seed):
    """Largest deviation of FP32 port runs on one-ulp perturbations of X from
    the FP64 pose (R, t): (degrees, x extent)."""
    rng = np.random.default_rng(seed)
    ext = float(np.ptp(np.asarray(X, np.float64), 0).max())
    dr = dt = 0.0
    for _ in range(C4_ENSEMBLE):
        Xp = np.asarray(X, np.float32) * (1 + rng.choice([-1, 0, 1], size=X.shape).astype(np.float32)
                                          * np.float32(6e-8))
        Re, te, _ = O.emicp(Xp.astype(np.float64), Y, precision="f32", trace=False, **EMICP)
        dr = max(dr, W.rotation_error_deg(Re, R))
        dt = max(dt, float(np.abs(te - t).max()) / ext)
    return dr, dt


def make_c4(with_reference=True):
    idx, sha, N, M, Rs, ts, Rps, tps, Rrs, trs, spr = [], [], [], [], [], [], [], [], [], [], []
    use_ref = with_reference and O.ref() is not None
    t0 = time.time()
    for k, (kind, X, Y, _, _) in enumerate(W.batch_pairs(count=256, seed=0)):
        if kind != "emicp":
            continue
        R, t, _ = O.emicp(X, Y, trace=False, **EMICP)
        Rp, tp, _ = O.emicp(X, Y, precision="f32", trace=False, **EMICP)
        if use_ref:
            Rr, tr_ = O.ref_emicp_cpu(X, Y, **EMICP)
            Rrs.append(Rr)
            trs.append(tr_)
        idx.append(k)
        sha.append(pair_sha(X, Y))
        N.append(len(X))
        M.append(len(Y))
        Rs.append(R)
        ts.append(t)
        Rps.append(Rp)
        tps.append(tp)
        spr.append(fp32_spread(X, Y, R, t, seed=1000 + k))
    print("c4 oracle f64: %d EM-ICP pairs, %.0f s" % (len(idx), time.time() - t0), flush=True)
    extra = dict(ref_R=np.array(Rrs), ref_t=np.array(trs)) if use_ref else {}
    np.savez_compressed(os.path.join(HERE, "c4_emicp_pairs.npz"), index=np.array(idx), sha=np.array(sha),
                        N=np.array(N), M=np.array(M), R=np.array(Rs), t=np.array(ts), port_R=np.array(Rps),
                        port_t=np.array(tps), spread=np.array(spr), **extra)


def main():
    which = [a for a in sys.argv[1:] if not a.startswith("--")] or ["c3", "c5", "c4", "c2"]
    O.set_threads(os.cpu_count() or 1)
    if "c3" in which:
        make_c3(with_reference="--no-reference" not in sys.argv)
    if "c5" in which:
        make_c5()
    if "c4" in which:
        make_c4(with_reference="--no-reference" not in sys.argv)
    if "c2" in which:
        make_c2()


if __name__ == "__main__":
    main()
