#!/usr/bin/env python
"""Benchmark of the soft-correspondence registration path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c3_emicp_40097|c1_emicp_1007|c2_softassign_2000|c5_softassign_20000|
                                icp_40097|c4_batch_256]

One step is one complete registration (the whole annealing schedule) of the
workload's seeded synthetic pair. The default workload is config 3: EM-ICP
with N = M = 40,097 (two ~70% views of a union of 3 ellipsoids, 5% uniform
outliers, rotation up to 20 degrees), the default schedule of 66 sigma steps.
Its points are the ones stored with the FP64 oracle's result in
tests/golden/c3_emicp_40097.npz, so the line can state the result's error
against that oracle ("accuracy").

ours:      `value` times the device-pointer C ABI entry point (inputs already
           in HBM) with CUDA events on the launching stream. L2 is flushed
           (256 MiB write) between steps, outside the timed events. `e2e`
           times the host-pointer entry point (pinned host SoA in, R,t out,
           copies included) by wall clock.
reference: times the reference's CPU implementation on the host cores: its own
           emicp_cpu() (src/emicp_cpu.cpp, compiled unmodified into
           oracle/_ref by oracle/build.py) for EM-ICP workloads, else the
           oracle's FP32 port of the reference algorithm (the reference has
           no CPU Softassign or exact ICP). Each step is a bounded sample of
           one registration: a whole number of sigma steps or pose updates of
           the full-size pair; `ms_per_step` is the time of that sample and
           `value` scales it to registrations/s.

c4_batch_256: one step is one batched launch (cesa_register_batch_device) of
the 256 pairs of config 4; value counts every pair as one registration. The
line also reports the same pairs registered one pair per launch.

Profiling cases: --size, --sigma-inf, --jmax, --i0 and --pairs run a smaller
case of a workload (same generator), and --no-cpu-baseline / --no-adjoint
skip the legs that are not being profiled. --timeline prints the in-kernel
phase timeline of one registration (EM-ICP or the banded Softassign form)
instead of a bench line.

Multi-GPU: one process per GPU (torchrun), independent replicas of the same
workload; value = registrations done by all ranks / max rank time.
Rank 0 prints one JSON line.
"""
import argparse
import copy
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

L2_FLUSH_BYTES = 256 << 20
GOLDEN = os.path.join(HERE, "tests", "golden")
DEFAULT_WORKLOAD = "c3_emicp_40097"
BATCH_WORKLOAD = "c4_batch_256"
ROT_BOUND_DEG = 1e-3
T_BOUND_REL = 1e-5


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0,
                    help="target seconds of CPU work for the CPU-baseline sample")
    ap.add_argument("--sinkhorn-form", default="auto", choices=["auto", "matrix_free", "materialised", "banded"],
                    help="Softassign Sinkhorn form (auto: the library's recorded choice for the size, "
                         "else its default by size)")
    ap.add_argument("--tune", action="store_true",
                    help="run the Sinkhorn autotuner for the workload's size before timing (records the "
                         "choice that auto then uses, and reports both forms' times)")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the forward + backward timing reported under 'adjoint'")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--size", type=int, default=None,
                    help="points per cloud (the workload's generator at a smaller size; profiling)")
    ap.add_argument("--sigma-inf", type=float, default=None, help="EM-ICP schedule end (profiling)")
    ap.add_argument("--jmax", type=int, default=None, help="Softassign JMAX (profiling)")
    ap.add_argument("--i0", type=int, default=None, help="Softassign I0 (profiling)")
    ap.add_argument("--pairs", type=int, default=256, help="pairs of the batch workload (profiling)")
    ap.add_argument("--iterations", type=int, default=None, help="ICP iterations (profiling)")
    ap.add_argument("--icp-search", default="auto", choices=["auto", "exhaustive", "grid"],
                    help="ICP nearest-neighbour search of the timed runs")
    ap.add_argument("--timeline", action="store_true",
                    help="print the in-kernel phase timeline of one registration instead of a bench line")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------ workload
class RefDefaults:
    """The reference CLI defaults (src/main.cpp:280-315), as FP32 values,
    without loading libcesa."""
    JMAX, I0, I1 = 100, 5, 3
    alpha = float(np.float32(3.0))
    T_0 = float(np.float32(100.0))
    TFACTOR = float(np.float32(0.95))
    moutlier = float(np.float32(np.exp(np.float32(-1.0)) / np.sqrt(np.float32(100.0))))
    sigma_p2 = float(np.float32(0.01))
    sigma_inf = float(np.float32(1e-5))
    sigma_factor = float(np.float32(0.9))
    d_02 = float(np.float32(0.01))
    maxIteration = 30


def schedule(args):
    """The workload's parameters: the reference defaults with the profiling
    overrides applied (identical in both arms)."""
    p = RefDefaults()
    if args.sigma_inf is not None:
        p.sigma_inf = float(np.float32(args.sigma_inf))
    if args.jmax is not None:
        p.JMAX = args.jmax
    if args.i0 is not None:
        p.I0 = args.i0
    if args.iterations is not None:
        p.maxIteration = args.iterations
    return p


def cesa_params(cesa, p, form="auto", icp_search="auto"):
    return cesa.Params.default(JMAX=p.JMAX, I0=p.I0, I1=p.I1, sigma_inf=p.sigma_inf, maxIteration=p.maxIteration,
                               sinkhorn_form=FORMS[form], icp_search=ICP_SEARCH[icp_search])


ICP_SEARCH = {"auto": 0, "exhaustive": 1, "grid": 2}


FORMS = {"auto": 0, "matrix_free": 1, "materialised": 2, "banded": 3}
FORM_NAMES = {1: "matrix_free", 2: "materialised", 3: "banded"}


def fixture_for(args, p):
    """The committed FP64-oracle fixture whose inputs and schedule are this
    run's, or None."""
    if args.size is not None or args.seed != 0:
        return None
    d = RefDefaults()
    if p.maxIteration != d.maxIteration:
        return None
    if args.workload == "c3_emicp_40097" and p.sigma_inf == d.sigma_inf:
        path = os.path.join(GOLDEN, "c3_emicp_40097.npz")
    elif args.workload == "c2_softassign_2000" and (p.JMAX, p.I0) == (d.JMAX, d.I0):
        path = os.path.join(GOLDEN, "c2_softassign_2000.npz")
    elif args.workload == "c5_softassign_20000" and p.JMAX == 2 and p.I0 == d.I0:
        path = os.path.join(GOLDEN, "c5_softassign_20000_jmax2.npz")
    else:
        return None
    return path if os.path.exists(path) else None


def load_workload(args, p):
    """(kind, X, Y, fixture) for the run: the fixture's stored points where
    one matches the run, else the seeded generator."""
    from cuda_emicp_softassign_gb300 import workloads as W
    kind, X, Y, _, _ = W.make(args.workload, seed=args.seed, n=args.size)
    fx = fixture_for(args, p)
    if fx is not None:
        g = np.load(fx)
        X, Y = g["X"], g["Y"]
    return kind, X, Y, fx


def pose_updates(kind, p):
    if kind == "softassign":
        return p.JMAX * p.I0
    if kind == "icp":
        return p.maxIteration
    return len(sigma_sequence(p))


def sigma_sequence(p):
    """sigma_p2 of every EM-ICP step (the reference's FP32 loop, src/emicp.cu:443,668)."""
    out, s = [], np.float32(p.sigma_p2)
    while s > np.float32(p.sigma_inf):
        out.append(float(s))
        s = np.float32(s * np.float32(p.sigma_factor))
    return out


def algorithmic_work(kind, N, M, p):
    """(fp32 ops, ex2 ops, affinity elements) of one registration.

    EM-ICP: per element 12 FP32-pipe ops + 1 ex2 (3 FADD, FMUL + 2 FFMA for
    d^2, FMUL scale, FFMA + FADD + 3 FFMA accumulators).
    ICP: per element and iteration 6 FP32-pipe ops (the squared distance) and a
    compare-select of (distance, index) on the ALU pipe, no ex2.
    Softassign: per pose update 2*I1 Sinkhorn sweeps of 8 FP32 ops + 1 ex2
    (3 FADD, FMUL + 2 FFMA, FFMA exponent, FFMA weighted sum) and one final
    sweep of 12 FP32 ops + 1 ex2 (the same with 5 weighted sums).
    These are the algorithm's counts; executed_work gives the kernels' own
    where they need fewer.
    """
    n = pose_updates(kind, p)
    e = float(N) * float(M)
    if kind == "emicp":
        return 12.0 * e * n, e * n, e * n
    if kind == "icp":
        return 6.0 * e * n, 0.0, e * n
    sweeps = 2 * p.I1
    return e * n * (8.0 * sweeps + 12.0), e * n * (sweeps + 1), e * n * (sweeps + 1)


def ranged_sweep(n_own, n_stream, grid):
    """Whether a sweep owning n_own points and streaming n_stream takes the
    ranged decomposition (at least 16 (128-point block, 512-point chunk) tasks
    per block of the persistent grid)."""
    return -(-n_own // 128) * -(-n_stream // 512) >= 16 * grid


def executed_work(kind, N, M, p, grid):
    """FP32-pipe ops the kernels execute for one registration, where they
    differ from the algorithmic count: the ranged EM-ICP sweep and the
    matrix-free Softassign sweeps run on clouds scaled by the exponent's
    factor (and fold 2^c0 into the streamed weights), so that the scale
    multiply is gone: EM-ICP 11 per element, Sinkhorn 7, final 11."""
    n = pose_updates(kind, p)
    e = float(N) * float(M)
    if kind == "emicp":
        return (11.0 if ranged_sweep(M, N, grid) else 12.0) * e * n
    return e * n * (7.0 * 2 * p.I1 + 11.0)


def materialised_bytes(N, M, p):
    """HBM bytes of one registration in the materialised form: per pose update
    4 B per element written (K) and 4 B read by each of the 2*I1 later passes."""
    return 4.0 * (1 + 2 * p.I1) * float(N) * float(M) * p.JMAX * p.I0


def kernels_per_registration(kind, form=None):
    # prep_center + 2 x prep_pack (+ 2 x fill for the slack vectors) + the persistent kernel;
    # the banded Softassign kernel initialises the slack itself
    if kind == "softassign" and form != "banded":
        return 6
    return 4


def config_of(args, kind, X, Y, p, fixture):
    c = {"workload": args.workload, "algorithm": kind, "N": int(len(X)), "M": int(len(Y)),
         "pose_updates_per_registration": pose_updates(kind, p), "seed": args.seed,
         "inputs": ("points stored in %s (the seeded generator's output)" % os.path.relpath(fixture, HERE)
                    if fixture else "seeded generator, cuda_emicp_softassign_gb300/workloads.py"),
         "l2": "flushed between steps (256 MiB write), outside the timed region",
         "parallelism": "replicas" if args.gpus > 1 else "single GPU"}
    if kind == "softassign":
        c.update(JMAX=p.JMAX, I0=p.I0, I1=p.I1, alpha=p.alpha, T_0=p.T_0, TFACTOR=p.TFACTOR)
    elif kind == "icp":
        c.update(maxIteration=p.maxIteration)
    else:
        c.update(sigma_p2=p.sigma_p2, sigma_inf=p.sigma_inf, sigma_factor=p.sigma_factor, d_02=p.d_02)
    return c


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # nvidia-smi takes a moment to start: wait (at most 5 s) for its first row, so that the
        # samples cover the timed region that follows rather than only its end.
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ CPU arm
def sigma_inf_after(p, k):
    """sigma_inf that makes the reference's loop run exactly its first k steps."""
    return sigma_sequence(p)[k - 1] * float(np.float32(p.sigma_factor)) if k > 0 else p.sigma_p2


def cpu_sample(kind, X, Y, p, target_s, threads=None):
    """One bounded sample of a registration on the host cores.

    EM-ICP: the reference's own emicp_cpu() where oracle/_ref built it (else
    the oracle's FP32 port), over the first k sigma steps of the schedule, k
    sized to about target_s. Softassign / ICP: the oracle's FP32 port over
    the first k pose updates (the reference has no CPU Softassign and its
    ICP needs FLANN). Returns dict(seconds, fraction, kind, impl, threads),
    fraction = the share of one registration the sample covers."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    O.set_threads(threads)
    n_full = pose_updates(kind, p)
    if kind == "emicp":
        use_ref = O.ref() is not None
        impl = ("the reference's own emicp_cpu() (src/emicp_cpu.cpp, FP32 + OpenBLAS, OpenMP), compiled "
                "unmodified by oracle/build.py" if use_ref else "the oracle's FP32 port of emicp_cpu() (OpenMP)")

        def run(k):
            si = sigma_inf_after(p, k)
            if use_ref:
                O.ref_emicp_cpu(X, Y, sigma_p2=p.sigma_p2, sigma_inf=si, sigma_factor=p.sigma_factor, d_02=p.d_02)
            else:
                O.emicp(X, Y, sigma_p2=p.sigma_p2, sigma_inf=si, sigma_factor=p.sigma_factor, d_02=p.d_02,
                        precision="f32", trace=False)
        unit, kind_out = "sigma steps", ("reference" if use_ref else "port")
    elif kind == "icp":
        impl = "the oracle's FP32 port of icp() with an exhaustive search (the reference's FLANN is absent)"

        def run(k):
            O.icp(X, Y, maxIteration=k, precision="f32", trace=False)
        unit, kind_out = "iterations", "port"
    else:
        impl = "the oracle's FP32 port of softassign() (OpenMP; the reference has no CPU Softassign)"

        def run(k):
            O.softassign(X, Y, JMAX=1, I0=k, I1=p.I1, alpha=p.alpha, T_0=p.T_0, TFACTOR=p.TFACTOR,
                         moutlier=p.moutlier, precision="f32", trace=False)
        unit, kind_out = "pose updates", "port"
    t0 = time.perf_counter()
    run(1)
    one = time.perf_counter() - t0
    k = int(max(1, min(n_full, round(target_s / max(one, 1e-6)))))
    if k == 1:
        dt = one
    else:
        t0 = time.perf_counter()
        run(k)
        dt = time.perf_counter() - t0
    return {"seconds": dt, "fraction": k / n_full, "kind": kind_out, "threads": threads,
            "sample": "first %d of the %d %s of one registration of the full-size pair: %s; scaled to a "
                      "registration by the share of the schedule it covers" % (k, n_full, unit, impl)}


def cpu_baseline(kind, X, Y, p, target_s):
    s = cpu_sample(kind, X, Y, p, target_s)
    return {"value": s["fraction"] / s["seconds"], "unit": "registrations/s", "cores": s["threads"],
            "kind": s["kind"], "sample": s["sample"]}


def run_reference(args, rank, world):
    if rank != 0:
        return
    if args.workload == BATCH_WORKLOAD:
        return run_reference_batch(args, world)
    p = schedule(args)
    kind, X, Y, fx = load_workload(args, p)
    per_step = max(0.5, args.cpu_sample_s / max(1, args.steps + args.warmup))
    secs, fracs = [], []
    t_all = time.perf_counter()
    for i in range(args.warmup + args.steps):
        s = cpu_sample(kind, X, Y, p, per_step)
        if i >= args.warmup:
            secs.append(s["seconds"])
            fracs.append(s["fraction"])
    value = float(np.sum(fracs) / np.sum(secs))
    line = {"impl": "reference", "metric": "registrations/s", "value": value, "unit": "registrations/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * float(np.mean(secs)),
            "registrations_per_step": float(np.mean(fracs)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_of(args, kind, X, Y, p, fx),
            "cpu_baseline": {"value": value, "unit": "registrations/s", "cores": s["threads"], "kind": s["kind"],
                             "sample": s["sample"]},
            "e2e": {"value": value, "unit": "registrations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t_all,
            "note": "each step is the sample named in cpu_baseline.sample (ms_per_step is its duration); value = "
                    "registrations covered by the timed samples / their total time"}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ accuracy
def accuracy(kind, X, Y, p, R, t, fixture):
    """Error of a registration against the FP64 oracle on the same inputs:
    the committed fixture where one matches, else the oracle run here when it
    is cheap (at most 2e10 affinity evaluations), else None."""
    from cuda_emicp_softassign_gb300 import workloads as W
    src = None
    if fixture:
        g = np.load(fixture)
        Ro, to = g["R"], g["t"]
        gap = float(g["trace"][-1, 30])
        src = "FP64 oracle (oracle/cesa_oracle.c), stored in %s" % os.path.relpath(fixture, HERE)
    else:
        _, _, elems = algorithmic_work(kind, len(X), len(Y), p)
        if elems > 2e10:
            return {"vs": None, "note": "the FP64 oracle is not run at this size here (%.2g affinity evaluations); "
                                        "the tests compare a cut schedule with a stored oracle result" % elems}
        from oracle import oracle as O
        O.set_threads(os.cpu_count() or 1)
        if kind == "emicp":
            Ro, to, tr = O.emicp(X, Y, sigma_p2=p.sigma_p2, sigma_inf=p.sigma_inf, sigma_factor=p.sigma_factor,
                                 d_02=p.d_02)
        elif kind == "softassign":
            Ro, to, tr = O.softassign(X, Y, JMAX=p.JMAX, I0=p.I0, I1=p.I1, alpha=p.alpha, T_0=p.T_0,
                                      TFACTOR=p.TFACTOR, moutlier=p.moutlier)
        else:
            Ro, to, tr, _ = O.icp(X, Y, maxIteration=p.maxIteration)
        gap = float(tr[-1, 30]) if len(tr) else None
        src = "FP64 oracle (oracle/cesa_oracle.c), run here on the same inputs"
    extent = float(np.ptp(np.asarray(X, np.float64), 0).max())
    e_r = W.rotation_error_deg(np.asarray(R, np.float64).reshape(3, 3), Ro)
    e_t = float(np.abs(np.asarray(t, np.float64) - to).max() / extent)
    return {"vs": src, "rot_err_deg": e_r, "t_err_over_extent": e_t, "bound_rot_deg": ROT_BOUND_DEG,
            "bound_t_over_extent": T_BOUND_REL, "within_bound": bool(e_r <= ROT_BOUND_DEG and e_t <= T_BOUND_REL),
            "horn_eigen_gap_final": gap}


# ------------------------------------------------------------------ helpers
def load_peaks():
    from cuda_emicp_softassign_gb300 import build
    L = ctypes.CDLL(build.PEAKS_LIB)
    L.cesa_peaks_measure.argtypes = [ctypes.POINTER(ctypes.c_double)] * 2
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    rc = L.cesa_peaks_measure(ctypes.byref(a), ctypes.byref(b))
    return (a.value, b.value) if rc == 0 else (None, None)


def max_over_ranks(values, world, device):
    """Element-wise maximum of this rank's timings over all ranks (each rank
    runs an independent replica; the slowest one sets the job time)."""
    import torch
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def whole_job_rate(steps, world, seconds):
    """Registrations per second of the whole job: every rank registers `steps`
    pairs, and the job takes the slowest rank's time."""
    return steps * world / seconds


def stored_traffic(roofline, key):
    """dram bytes per launch of the workload's kernel from a stored ncu capture
    (profiles/ncu_traffic.json, summarised in profiles/*.md). ncu cannot run
    inside the bench, so this figure is copied from that capture, not
    measured in this run; the line says so."""
    path = os.path.join(HERE, "profiles", "ncu_traffic.json")
    if not os.path.exists(path):
        return
    entry = json.load(open(path)).get(key)
    if entry:
        roofline["traffic"] = entry["bytes_per_launch"]
        roofline["traffic_source"] = ("copied from a stored ncu capture (profiles/ncu_traffic.json, %s), "
                                      "not measured in this run" % entry.get("profile", "profiles/"))


# ------------------------------------------------------------------ batch
def batch_schedules(args):
    """(EM-ICP, Softassign) parameters of the batch's pairs: the defaults, and
    JMAX = 60 for Softassign (config 4), with the profiling overrides."""
    em, sa = RefDefaults(), RefDefaults()
    sa.JMAX = 60
    if args.sigma_inf is not None:
        em.sigma_inf = float(np.float32(args.sigma_inf))
    if args.jmax is not None:
        sa.JMAX = args.jmax
    if args.i0 is not None:
        sa.I0 = args.i0
    return em, sa


def batch_workload(args):
    """Config 4: 256 pairs, N and M log-uniform in [500, 20000], config-1
    generator per pair; even pairs EM-ICP (default parameters), odd pairs
    Softassign (config-2 parameters, JMAX = 60). --pairs keeps the first
    pairs."""
    import cuda_emicp_softassign_gb300 as cesa
    from cuda_emicp_softassign_gb300 import workloads as W
    em, sa = batch_schedules(args)
    out = []
    for kind, X, Y, _, _ in W.batch_pairs(count=256, seed=args.seed)[:args.pairs]:
        if kind == "emicp":
            out.append((cesa.ALGO_EMICP, X, Y, cesa_params(cesa, em)))
        else:  # the form applies to the one-pair-per-launch comparison (the batch runs its own sweeps)
            out.append((cesa.ALGO_SOFTASSIGN, X, Y, cesa_params(cesa, sa, args.sinkhorn_form)))
    return out


def batch_pairs_cpu(args):
    """The config-4 pairs without loading libcesa: (algorithm, X, Y, params)."""
    from cuda_emicp_softassign_gb300 import workloads as W
    em, sa = batch_schedules(args)
    out = []
    for kind, X, Y, _, _ in W.batch_pairs(count=256, seed=args.seed)[:args.pairs]:
        out.append((0, X, Y, em) if kind == "emicp" else (1, X, Y, sa))
    return out


def batch_work(pairs):
    """(fp32 ops, ex2 ops, affinity elements) of one batched registration of all pairs."""
    f = x = e = 0.0
    for algo, X, Y, p in pairs:
        kind = "emicp" if algo == 0 else "softassign"
        a, b, c = algorithmic_work(kind, len(X), len(Y), p)
        f, x, e = f + a, x + b, e + c
    return f, x, e


def batch_config(args, pairs):
    n = [len(X) for _, X, _, _ in pairs]
    m = [len(Y) for _, _, Y, _ in pairs]
    em, sa = batch_schedules(args)
    return {"workload": BATCH_WORKLOAD, "pairs": len(pairs),
            "emicp_pairs": sum(1 for a, _, _, _ in pairs if a == 0),
            "softassign_pairs": sum(1 for a, _, _, _ in pairs if a == 1),
            "N_range": [int(min(n)), int(max(n))], "M_range": [int(min(m)), int(max(m))],
            "emicp_sigma_inf": em.sigma_inf, "softassign_JMAX": sa.JMAX, "softassign_I0": sa.I0, "seed": args.seed,
            "l2": "flushed between steps (256 MiB write), outside the timed region",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


def batch_cpu_sample(pairs, target_s):
    """One bounded CPU sample of the batch: the first pose updates of the
    first pairs (EM-ICP through the reference's own emicp_cpu() where built,
    Softassign through the FP32 port), timed per affinity element and scaled
    to the batch's total elements. Returns (registrations/s, seconds, desc,
    kind, threads)."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    use_ref = O.ref() is not None
    _, _, total = batch_work(pairs)
    spent = elems = 0.0
    used = 0
    for algo, X, Y, p in pairs:
        if spent > target_s:
            break
        t0 = time.perf_counter()
        if algo == 0:
            si = sigma_inf_after(p, 6)
            if use_ref:
                O.ref_emicp_cpu(X, Y, sigma_p2=p.sigma_p2, sigma_inf=si, sigma_factor=p.sigma_factor, d_02=p.d_02)
            else:
                O.emicp(X, Y, sigma_p2=p.sigma_p2, sigma_inf=si, sigma_factor=p.sigma_factor, d_02=p.d_02,
                        precision="f32", trace=False)
            elems += float(len(X)) * len(Y) * 6
        else:
            O.softassign(X, Y, JMAX=1, I0=1, I1=p.I1, alpha=p.alpha, T_0=p.T_0, TFACTOR=p.TFACTOR,
                         moutlier=p.moutlier, precision="f32", trace=False)
            elems += float(len(X)) * len(Y) * (2 * p.I1 + 1)
        spent += time.perf_counter() - t0
        used += 1
    per_elem = spent / elems
    regs = len(pairs) / (per_elem * total)
    desc = ("first pose updates of %d of the %d pairs (EM-ICP: %s; Softassign: the FP32 port): %.3g s per affinity "
            "element, scaled to the batch's %.3g elements"
            % (used, len(pairs), "the reference's own emicp_cpu()" if use_ref else "the FP32 port", per_elem, total))
    return regs, spent, desc, ("reference+port" if use_ref else "port"), threads


def run_reference_batch(args, world):
    pairs = batch_pairs_cpu(args)
    per_step = max(0.5, args.cpu_sample_s / max(1, args.steps + args.warmup))
    secs, regs = [], []
    for i in range(args.warmup + args.steps):
        v, dt, desc, kind, thr = batch_cpu_sample(pairs, per_step)
        if i >= args.warmup:
            secs.append(dt)
            regs.append(v * dt)
    value = float(np.sum(regs) / np.sum(secs))
    line = {"impl": "reference", "metric": "registrations/s", "value": value, "unit": "registrations/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(secs)),
            "registrations_per_step": float(np.mean(regs)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": batch_config(args, pairs),
            "cpu_baseline": {"value": value, "unit": "registrations/s", "cores": thr, "kind": kind, "sample": desc},
            "e2e": {"value": value, "unit": "registrations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batch(args, rank, world, local):
    """Config 4: one step = one batched registration of all 256 pairs
    (cesa_register_batch_device, inputs resident). Also reported: the same
    pairs registered one pair per launch with the single-pair kernels."""
    import torch
    import cuda_emicp_softassign_gb300 as cesa

    torch.cuda.set_device(local)
    pairs = batch_workload(args)
    dev = []
    pose0 = torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")
    for algo, X, Y, p in pairs:
        dX = torch.from_numpy(cesa.cloud2data(X)).cuda()
        dY = torch.from_numpy(cesa.cloud2data(Y)).cuda()
        dev.append([algo, dX, dY, pose0.clone(), p])
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def reset():
        for d in dev:
            d[3].copy_(pose0)

    for _ in range(args.warmup):
        flush.zero_()
        reset()
        cesa.register_batch_device([tuple(d) for d in dev], d_status=status, stream=stream)
    torch.cuda.synchronize()
    assert cesa.stream_status(stream) == 0
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        reset()
        ev[k][0].record(stream)
        cesa.register_batch_device([tuple(d) for d in dev], d_status=status, stream=stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    assert cesa.stream_status(stream) == 0 and int(status.item()) == 0
    total_ms = float(np.sum([a.elapsed_time(b) for a, b in ev]))

    # the same pairs, one pair per launch (single-pair device entry points); per pair the time of
    # its own launch sequence, so that the sum of the pairs' latency floors is known too
    single_ms = 0.0
    per_pair_ms = []
    for algo, dX, dY, dRt, p in dev:
        dRt.copy_(pose0)
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        (cesa.emicp_device if algo == 0 else cesa.softassign_device)(dX, dY, dRt, param=p, d_status=status,
                                                                      stream=stream)
        e1.record(stream)
        e1.synchronize()
        per_pair_ms.append(e0.elapsed_time(e1))
        single_ms += per_pair_ms[-1]

    # end to end through the host-pointer batch entry point
    e2e_steps = max(1, min(args.steps, 3))
    cesa.register_batch(pairs)
    e2e_s = 0.0
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cesa.register_batch(pairs)
        e2e_s += time.perf_counter() - t0
    e2e_s /= e2e_steps

    total_ms, e2e_s, single_ms = max_over_ranks([total_ms, e2e_s, single_ms], world, "cuda")
    if rank != 0:
        return
    npairs = len(pairs)
    mean_s = total_ms * 1e-3 / args.steps
    value = whole_job_rate(args.steps * npairs, world, total_ms * 1e-3)
    fp32_ops, ex2_ops, elems = batch_work(pairs)
    fp32_peak, ex2_peak = load_peaks()
    achieved = fp32_ops / mean_s / 1e12
    roofline = {"bound": "fp32", "kernel": "batch_kernel", "achieved": achieved,
                "peak": fp32_peak / 1e12 if fp32_peak else None, "unit": "TFLOP/s",
                "frac": achieved / (fp32_peak / 1e12) if fp32_peak else None, "traffic": None,
                "peak_source": "measured in this run: FFMA lane-op rate (libcesa_peaks), FMA counted as 1 op",
                "ex2_achieved_tops": ex2_ops / mean_s / 1e12,
                "ex2_peak_tops": ex2_peak / 1e12 if ex2_peak else None,
                "ops_per_batch": fp32_ops}
    # Lower bound of the batch's time: the work at the measured FP32 peak, and no pair can finish
    # faster than its own latency floor (its single-pair launch, which already runs at or near the
    # peak for large pairs). The batch cannot beat max(total work / peak, longest single pair).
    work_s = fp32_ops / fp32_peak if fp32_peak else None
    longest = max(per_pair_ms) * 1e-3
    bound_s = max(work_s or 0.0, longest)
    cpu = None
    if not args.no_cpu_baseline:
        v, dt, desc, kind, thr = batch_cpu_sample(pairs, args.cpu_sample_s)
        cpu = {"value": v, "unit": "registrations/s", "cores": thr, "kind": kind, "sample": desc}
    h2d = sum((len(X) + len(Y)) * 3 * 4 + 48 for _, X, Y, _ in pairs)
    line = {"metric": "registrations/s", "value": value, "unit": "registrations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator of config 4; see cuda_emicp_softassign_gb300/workloads.py)",
            "config": batch_config(args, pairs),
            "gelem_per_s": elems * args.steps * world / (total_ms * 1e-3) / 1e9,
            "one_pair_per_launch": {"value": world * npairs / (single_ms * 1e-3), "unit": "registrations/s",
                                    "ms": single_ms, "batched_speedup": single_ms / (total_ms / args.steps)},
            "batch_time_bound": {"ms": bound_s * 1e3, "work_at_fp32_peak_ms": work_s * 1e3 if work_s else None,
                                 "longest_single_pair_ms": longest * 1e3,
                                 "max_speedup_vs_one_pair_per_launch": single_ms * 1e-3 / bound_s,
                                 "note": "the batch cannot finish before its FP32 work at the measured peak, "
                                         "nor before its longest pair alone"},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": world * npairs / e2e_s, "unit": "registrations/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 48 * npairs},
            "clocks": clocks,
            "gpu_launches": 3 * args.steps,
            "wall_s_timed_region": t_wall}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ adjoint
def measure_adjoint(cesa, kind, dX, dY, N, M, p, pose0, reps=3):
    """Forward + adjoint (cesa_<kind>_forward_device then
    cesa_<kind>_backward_device for the loss |R - I|^2 + |t|^2), CUDA events.
    Returns the plain forward, taped forward and backward milliseconds (best of
    reps) and (taped forward + backward) / plain forward. Softassign's taped
    forward runs the matrix-free kernel, so its plain forward is timed in that
    form too."""
    import torch
    L = cesa.lib()
    tape_bytes = getattr(L, "cesa_%s_tape_bytes" % kind)
    fwd = getattr(L, "cesa_%s_forward_device" % kind)
    bwd = getattr(L, "cesa_%s_backward_device" % kind)
    plain = cesa.emicp_device if kind == "emicp" else cesa.softassign_device
    if kind == "softassign":
        p = copy.copy(p)
        p.sinkhorn_form = cesa.SINKHORN_MATRIX_FREE
    nbytes = tape_bytes(N, M, ctypes.byref(p))
    tape = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    dRt = pose0.clone()
    g = torch.empty(12, dtype=torch.float32, device="cuda")
    gX = torch.empty(3 * N, dtype=torch.float32, device="cuda")
    gY = torch.empty(3 * M, dtype=torch.float32, device="cuda")
    g0 = torch.empty(12, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    sh = ctypes.c_void_p(st.cuda_stream)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    best = [1e30, 1e30, 1e30]
    for _ in range(reps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        dRt.copy_(pose0)
        ev[0].record(st)
        plain(dX, dY, dRt, param=p, stream=st)
        ev[1].record(st)
        dRt.copy_(pose0)
        ev[2].record(st)
        assert fwd(ptr(dX), N, ptr(dY), M, ptr(dRt), ctypes.byref(p), ptr(tape), None, sh) == 0
        ev[3].record(st)
        g.copy_(2.0 * (dRt - pose0))  # d/d(R, t) of |R - I|^2 + |t|^2
        st.synchronize()
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e4.record(st)
        assert bwd(N, M, ctypes.byref(p), ptr(tape), ptr(g), ptr(gX), ptr(gY), ptr(g0), None, sh) == 0
        e5.record(st)
        st.synchronize()
        best = [min(best[0], ev[0].elapsed_time(ev[1])), min(best[1], ev[2].elapsed_time(ev[3])),
                min(best[2], e4.elapsed_time(e5))]
    note = ("taped forward records pose, moments, Horn eigenbasis and per-row C, lambda, u per step; "
            "the backward recomputes the affinities (no N x M storage)") if kind == "emicp" else \
        ("taped forward (matrix-free) records every Sinkhorn pass's scalings and sums; the backward recomputes "
         "the affinities in each K product (no N x M storage)")
    return {"fwd_ms": best[0], "fwd_taped_ms": best[1], "bwd_ms": best[2],
            "fwd_plus_bwd_over_fwd": (best[1] + best[2]) / best[0], "tape_bytes": int(nbytes),
            "loss": "|R - I|_F^2 + |t|^2 of the registered pose", "note": note}


# ------------------------------------------------------------------ timeline
TL_NAMES = {
    "emicp": {1: "start", 2: "a unit's first chunk landed", 3: "unit swept", 4: "unit's row partials stored",
              5: "grid barrier after the sweep", 8: "rows completed, block moments, grid barrier",
              6: "moment records reduced", 7: "S (nine threads) + pose solve"},
    "softassign": {1: "start", 2: "final: last column pass completed", 3: "row pass completed (cluster)",
                   4: "column sweep + partial store (final: record store)",
                   5: "barrier (column tile's CTAs; the grid before the pose)", 6: "moment records reduced",
                   7: "Horn solve", 8: "cluster barrier (final sweep included after 2)",
                   10: "moments: cluster barrier", 11: "final rows finalised", 12: "moments summed",
                   13: "S formed", 14: "column pass completed (band partials)", 15: "row sweep + warp reduction"},
}


def run_timeline(args):
    """Mean duration of each phase of a pose update in block 0 of the
    persistent grid (the library's %globaltimer timeline, cesa_report), and
    for Softassign how many updates the certified pose solve took."""
    import cuda_emicp_softassign_gb300 as cesa
    p = schedule(args)
    kind, X, Y, _ = load_workload(args, p)
    form = "banded" if (kind == "softassign" and args.sinkhorn_form == "auto") else args.sinkhorn_form
    q = cesa_params(cesa, p, form)
    fn = cesa.emicp if kind == "emicp" else cesa.softassign
    _, _, tr, _ = fn(X, Y, param=q, trace=True)
    cap = 320 * 40 * max(1, pose_updates(kind, p))  # blocks x entries per update x updates
    _, _, tl, rep = fn(X, Y, param=q, timeline=cap)
    rows = cesa.timeline_table(tl, rep.grid_blocks)
    b0 = rows[rows[:, 0] == 0][:, 1:]
    starts = np.where(b0[:, 0] == 1)[0]
    segs = [b0[a:b + 1] for a, b in zip(starts[1:-1], starts[2:])]
    segs = [sg for sg in segs if len(sg) == len(segs[0])]
    names = TL_NAMES["emicp" if kind == "emicp" else "softassign"]
    out = {"workload": args.workload, "N": len(X), "M": len(Y), "grid_blocks": rep.grid_blocks,
           "sinkhorn_form": FORM_NAMES.get(rep.sinkhorn_form) if kind == "softassign" else None,
           "updates_in_mean": len(segs),
           "ns_per_update": float(np.mean([sg[-1, 1] - sg[0, 1] for sg in segs])), "phases": []}
    for i in range(1, len(segs[0])):
        out["phases"].append((names.get(int(segs[0][i, 0]), "next update"),
                              float(np.mean([sg[i, 1] - sg[i - 1, 1] for sg in segs]))))
    if len(tr):
        out["certified_pose_solves"] = int((tr[:, 30] == -1).sum())
    print(json.dumps(out), flush=True)


# ------------------------------------------------------------------ ours
def run_ours(args, rank, world, local):
    import torch
    import torch.distributed as dist
    import cuda_emicp_softassign_gb300 as cesa

    torch.cuda.set_device(local)
    sp = schedule(args)
    kind, X, Y, fx = load_workload(args, sp)
    p = cesa_params(cesa, sp, args.sinkhorn_form, args.icp_search)
    N, M = len(X), len(Y)
    tuned = None
    if kind == "softassign" and args.tune:
        f, ms_free, ms_mat = cesa.tune_sinkhorn(N, M, p)  # records the choice used by "auto"
        tuned = {"chosen": FORM_NAMES.get(f, "matrix_free"),
                 "ms_per_update_matrix_free": ms_free, "ms_per_update_materialised": ms_mat}
    dev_call = {"emicp": cesa.emicp_device, "softassign": cesa.softassign_device, "icp": cesa.icp_device}[kind]

    dX = torch.from_numpy(cesa.cloud2data(X)).cuda()
    dY = torch.from_numpy(cesa.cloud2data(Y)).cuda()
    pose0 = torch.tensor(np.r_[np.eye(3).reshape(-1), np.zeros(3)], dtype=torch.float32, device="cuda")
    dRt = pose0.clone()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        flush.zero_()
        dRt.copy_(pose0)
        dev_call(dX, dY, dRt, param=p, d_status=status, stream=stream)
    torch.cuda.synchronize()
    assert cesa.stream_status(stream) == 0
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()

    sampler = ClockSampler(torch.cuda.current_device())
    sampler.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        dRt.copy_(pose0)
        ev[k][0].record(stream)
        dev_call(dX, dY, dRt, param=p, d_status=status, stream=stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clocks = sampler.stop()
    st = cesa.stream_status(stream)
    assert st == 0, "device status %d" % st
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = float(np.sum(step_ms))
    R_dev = dRt.cpu().numpy().astype(np.float64)

    # ---- end to end through the host-pointer C ABI (pinned SoA in, R,t out)
    hX = torch.from_numpy(cesa.cloud2data(X)).pin_memory().numpy()
    hY = torch.from_numpy(cesa.cloud2data(Y)).pin_memory().numpy()
    lib = cesa.lib()
    Rh = np.eye(3, dtype=np.float32).reshape(-1).copy()
    th = np.zeros(3, np.float32)
    fn = {"emicp": lib.cesa_emicp, "softassign": lib.cesa_softassign, "icp": lib.cesa_icp}[kind]
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    for _ in range(max(1, args.warmup)):
        Rh[:] = np.eye(3, dtype=np.float32).reshape(-1)
        th[:] = 0
        assert fn(ptr(hX), N, ptr(hY), M, ptr(Rh), ptr(th), ctypes.byref(p), None) == 0
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        Rh[:] = np.eye(3, dtype=np.float32).reshape(-1)
        th[:] = 0
        t0 = time.perf_counter()
        rc = fn(ptr(hX), N, ptr(hY), M, ptr(Rh), ptr(th), ctypes.byref(p), None)
        e2e_s += time.perf_counter() - t0
        assert rc == 0
    assert np.array_equal(Rh.astype(np.float64), R_dev[:9]), "host and device entry points disagree"

    # ---- max over ranks
    total_ms, e2e_s = max_over_ranks([total_ms, e2e_s], world, "cuda")
    if rank != 0:
        return

    regs = args.steps * world
    value = whole_job_rate(args.steps, world, total_ms * 1e-3)
    fp32_ops, ex2_ops, elems = algorithmic_work(kind, N, M, sp)
    mean_s = total_ms * 1e-3 / args.steps
    fp32_peak, ex2_peak = load_peaks()
    achieved = fp32_ops / mean_s / 1e12
    roofline = {"bound": "fp32", "kernel": "%s_kernel" % kind,
                "achieved": achieved, "peak": fp32_peak / 1e12 if fp32_peak else None, "unit": "TFLOP/s",
                "frac": achieved / (fp32_peak / 1e12) if fp32_peak else None,
                "traffic": None,
                "peak_source": "measured in this run: FFMA lane-op rate (libcesa_peaks), FMA counted as 1 op; "
                               "MEASURED_PEAKS.json carries no FP32/MUFU figure",
                "ex2_achieved_tops": ex2_ops / mean_s / 1e12,
                "ex2_peak_tops": ex2_peak / 1e12 if ex2_peak else None,
                "ops_per_registration": fp32_ops,
                "note": "achieved = algorithmic FP32-pipe ops of one registration / event time of its launch "
                        "sequence (prep kernels included); executed_fp32_ops_per_registration, where given, "
                        "is what the kernels issue on the FP32 pipe (clouds pre-scaled by the exponent's "
                        "factor, one op fewer per element)"}
    form_used = None
    if kind == "softassign":
        # the form the library resolved for this request (AUTO: tuned or by size), as it reports it
        q = copy.copy(p)
        q.JMAX = 1
        rep = cesa.softassign(X, Y, param=q, trace=True)[3]
        form_used = FORM_NAMES.get(rep.sinkhorn_form, str(rep.sinkhorn_form))
        if form_used == "matrix_free":
            roofline["executed_fp32_ops_per_registration"] = executed_work(kind, N, M, sp, rep.grid_blocks)
    if kind == "emicp":
        q = copy.copy(p)
        q.sigma_inf = q.sigma_p2 * 0.95  # one sigma step: the plan and grid of this size
        rep = cesa.emicp(X, Y, param=q, trace=True)[3]
        roofline["executed_fp32_ops_per_registration"] = executed_work(kind, N, M, sp, rep.grid_blocks)
    if form_used == "banded":
        roofline["note"] += (". The banded form computes each affinity once per inner iteration and "
                             "keeps the tile in shared memory for the other 2*I1 sweeps, so it executes "
                             "fewer operations than this per-sweep count: per element and pose update 1 ex2 "
                             "and %d FP32 ops (the first row sweep 8, each later Sinkhorn sweep 1, the final "
                             "sweep 5)" % (8 + (2 * sp.I1 - 1) + 5))
        roofline["kernel"] = "softassign_band_kernel"
        roofline["executed_fp32_ops_per_registration"] = float(N) * float(M) * pose_updates(kind, sp) * (
            8 + (2 * sp.I1 - 1) + 5)
    if form_used == "materialised":
        hbm_peak = None
        try:
            hbm_peak = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))["hbm_gbs"]
        except (OSError, KeyError, ValueError):
            pass
        gbs = materialised_bytes(N, M, sp) / mean_s / 1e9
        roofline = {"bound": "hbm", "kernel": "softassign_mat_kernel", "achieved": gbs,
                    "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak if hbm_peak else None,
                    "traffic": None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)",
                    "bytes_per_registration": materialised_bytes(N, M, sp),
                    "note": "achieved = algorithmic HBM bytes (4 B per element written once and read by "
                            "each of the 2*I1 later passes, per pose update) / event time"}
    if args.size is None and args.sigma_inf is None and args.jmax is None and args.i0 is None:
        stored_traffic(roofline, args.workload + (":" + form_used if form_used in ("materialised", "banded") else ""))
    cpu = None if args.no_cpu_baseline else cpu_baseline(kind, X, Y, sp, args.cpu_sample_s)
    acc = accuracy(kind, X, Y, sp, R_dev[:9], R_dev[9:12], fx)
    h2d = (N + M) * 3 * 4 + 12 * 4
    line = {"metric": "registrations/s", "value": value, "unit": "registrations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator of the workload; see cuda_emicp_softassign_gb300/workloads.py)",
            "config": config_of(args, kind, X, Y, sp, fx),
            "accuracy": acc,
            "gelem_per_s": elems * regs / (total_ms * 1e-3) / 1e9,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": whole_job_rate(args.steps, world, e2e_s), "unit": "registrations/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 12 * 4},
            "clocks": clocks,
            "gpu_launches": kernels_per_registration(kind, form_used) * args.steps,
            "wall_s_timed_region": t_wall}
    if kind == "softassign":
        line["sinkhorn"] = {"form": form_used, "requested": args.sinkhorn_form, "tuner": tuned}
    if kind == "icp":
        # value is the default search (a uniform grid from 4096 target points on), whose work depends
        # on the data; the FP32 roofline is that of the exhaustive search, timed here on the same pair
        pe = copy.copy(p)
        pe.icp_search = cesa.ICP_SEARCH_EXHAUSTIVE
        exh = []
        for k in range(max(2, args.steps)):
            flush.zero_()
            dRt.copy_(pose0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            cesa.icp_device(dX, dY, dRt, param=pe, d_status=status, stream=stream)
            b.record(stream)
            torch.cuda.synchronize()
            if k > 0:
                exh.append(a.elapsed_time(b))
        exh_s = float(np.mean(exh)) * 1e-3
        achieved = fp32_ops / exh_s / 1e12
        roofline.update({"kernel": "icp_kernel (exhaustive search)", "achieved": achieved,
                         "frac": achieved / (fp32_peak / 1e12) if fp32_peak else None})
        roofline["note"] = ("achieved = 6 FP32-pipe ops per point pair (squared distance; the compare-select "
                            "of (distance, index) runs on the ALU pipe) x N x M x iterations / event time of "
                            "the exhaustive search on the same pair")
        used = args.icp_search if args.icp_search != "auto" else ("grid" if N >= 4096 else "exhaustive")
        line["icp_search"] = {"value_search": used,
                              "ms_per_step": total_ms / args.steps, "exhaustive_ms_per_step": exh_s * 1e3,
                              "note": "both searches are exact and return the same matches"}
    if not args.no_adjoint and kind != "icp":
        adj = measure_adjoint(cesa, kind, dX, dY, N, M, p, pose0)
        if kind == "emicp":
            # the backward's own roofline: 19 FP32-pipe ops per element and sigma step
            fp32_peak, _ = load_peaks()
            ops = 19.0 * float(N) * float(M) * pose_updates(kind, p)
            ach = ops / (adj["bwd_ms"] * 1e-3) / 1e12
            adj["roofline"] = {
                "bound": "fp32", "kernel": "emicp_adjoint_kernel", "achieved": ach,
                "peak": fp32_peak / 1e12 if fp32_peak else None, "unit": "TFLOP/s",
                "frac": ach / (fp32_peak / 1e12) if fp32_peak else None,
                "executed_fp32_ops_per_registration": ops,
                "note": ("19 FP32-pipe ops per affinity element and sigma step, executed as packed pairs (6 for "
                         "the distance, 4 for ge, 3 for t = gB - ge (x - z) / s2, 3 each for dL/dx and dL/dz "
                         "+= e t), over the N x M elements without padding, divided by the backward call's "
                         "event time; peak as the forward's")}
        if kind == "softassign" and form_used != "matrix_free":
            # the tape comes from the matrix-free kernel; against the forward this
            # request actually runs (value's form) the ratio is higher
            fwd_auto = total_ms / args.steps
            adj["fwd_%s_ms" % form_used] = fwd_auto
            adj["fwd_plus_bwd_over_fwd_%s" % form_used] = (adj["fwd_taped_ms"] + adj["bwd_ms"]) / fwd_auto
        line["adjoint"] = adj
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.timeline:
        return run_timeline(args)
    if world > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "ours":
            torch.cuda.set_device(local)
        dist.init_process_group(backend="nccl" if (args.impl == "ours" and torch.cuda.is_available()) else "gloo")
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        elif args.workload == BATCH_WORKLOAD:
            run_batch(args, rank, world, local)
        else:
            run_ours(args, rank, world, local)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
