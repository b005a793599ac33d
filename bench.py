#!/usr/bin/env python
"""Benchmark of the soft-correspondence registration path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c2_softassign_2000|c1_emicp_1007|c3_emicp_40097|c5_softassign_20000|icp_40097|
                                c4_batch_256]

One step is one complete registration (the whole annealing schedule) of the
workload's seeded synthetic pair. The default workload is config 2: Softassign
with N ~ M ~ 2000 and JMAX=100, I0=5, I1=3, i.e. 500 pose updates.

ours:      `value` times the device-pointer C ABI entry point (inputs already
           in HBM) with CUDA events on the launching stream. L2 is flushed
           (256 MiB write) between steps, outside the timed events. `e2e`
           times the host-pointer entry point (pinned host SoA in, R,t out,
           copies included) by wall clock.
reference: times the reference algorithm on the host cores (the oracle's FP32
           port of the path, all threads) on a bounded sample of the same
           workload, scaled to registrations/s.

c4_batch_256: one step is one batched launch (cesa_register_batch_device) of
the 256 pairs of config 4; value counts every pair as one registration. The
line also reports the same pairs registered one pair per launch.

Multi-GPU: one process per GPU (torchrun), independent replicas of the same
workload; value = registrations done by all ranks / max rank time.
Rank 0 prints one JSON line.
"""
import argparse
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


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2_softassign_2000")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0,
                    help="target seconds of CPU work for the CPU-baseline sample")
    ap.add_argument("--sinkhorn-form", default="auto", choices=["auto", "matrix_free", "materialised", "banded"],
                    help="Softassign Sinkhorn form (auto: the library's recorded choice for the size, "
                         "matrix-free when none)")
    ap.add_argument("--tune", action="store_true",
                    help="run the Sinkhorn autotuner for the workload's size before timing (records the "
                         "choice that auto then uses, and reports both forms' times)")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the forward + backward timing reported under 'adjoint'")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(name, seed):
    from cuda_emicp_softassign_gb300 import workloads as W
    kind, X, Y, Rt, tt = W.make(name, seed=seed)
    return kind, X, Y


class RefDefaults:
    """The reference CLI defaults (src/main.cpp:280-315), without loading libcesa."""
    JMAX, I0, I1, alpha, T_0, TFACTOR = 100, 5, 3, 3.0, 100.0, 0.95
    moutlier = float(np.float32(np.exp(np.float32(-1.0)) / np.sqrt(np.float32(100.0))))
    sigma_p2, sigma_inf, sigma_factor, d_02 = 0.01, 1e-5, 0.9, 0.01
    maxIteration = 30


FORMS = {"auto": 0, "matrix_free": 1, "materialised": 2, "banded": 3}
FORM_NAMES = {1: "matrix_free", 2: "materialised", 3: "banded"}


def params_for(cesa, kind, form="auto"):
    return cesa.Params.default(sinkhorn_form=FORMS[form])


def materialised_bytes(N, M, p):
    """HBM bytes of one registration in the materialised form: per pose update
    4 B per element written (K) and 4 B read by each of the 2*I1 later passes."""
    return 4.0 * (1 + 2 * p.I1) * float(N) * float(M) * p.JMAX * p.I0


def pose_updates(kind, p):
    if kind == "softassign":
        return p.JMAX * p.I0
    if kind == "icp":
        return p.maxIteration
    n, s = 0, np.float32(p.sigma_p2)
    while s > np.float32(p.sigma_inf):
        n += 1
        s = np.float32(s * np.float32(p.sigma_factor))
    return n


def algorithmic_work(kind, N, M, p):
    """(fp32 ops, ex2 ops, affinity elements) of one registration.

    EM-ICP: per element 12 FP32-pipe ops + 1 ex2 (3 FADD, FMUL + 2 FFMA for
    d^2, FMUL scale, FFMA + FADD + 3 FFMA accumulators).
    ICP: per element and iteration 6 FP32-pipe ops (the squared distance) and a
    compare-select of (distance, index) on the ALU pipe, no ex2.
    Softassign: per pose update 2*I1 Sinkhorn sweeps of 8 FP32 ops + 1 ex2
    (3 FADD, FMUL + 2 FFMA, FFMA exponent, FFMA weighted sum) and one final
    sweep of 12 FP32 ops + 1 ex2 (the same with 5 weighted sums).
    """
    n = pose_updates(kind, p)
    e = float(N) * float(M)
    if kind == "emicp":
        return 12.0 * e * n, e * n, e * n
    if kind == "icp":  # 3 FADD, FMUL + 2 FFMA per element; the compare-select runs on the ALU pipe
        return 6.0 * e * n, 0.0, e * n
    sweeps = 2 * p.I1
    return e * n * (8.0 * sweeps + 12.0), e * n * (sweeps + 1), e * n * (sweeps + 1)


def kernels_per_registration(kind, form=None):
    # prep_center + 2 x prep_pack (+ 2 x fill for the slack vectors) + the persistent kernel;
    # the banded Softassign kernel initialises the slack itself
    if kind == "softassign" and form != "banded":
        return 6
    return 4


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


def cpu_baseline(kind, X, Y, p, target_s, threads=None):
    """Times the oracle's FP32 port of the reference algorithm on the host on a
    bounded sample; returns (registrations/s, description, threads)."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    O.set_threads(threads)
    n_full = pose_updates(kind, p)
    # calibrate with one pose update, then size the sample to ~target_s
    if kind == "emicp":
        s1 = np.float32(p.sigma_p2) * np.float32(p.sigma_factor)
        t0 = time.perf_counter()
        O.emicp(X, Y, sigma_p2=p.sigma_p2, sigma_inf=float(s1), sigma_factor=p.sigma_factor,
                d_02=p.d_02, precision="f32", trace=False)
        one = time.perf_counter() - t0
        k = int(max(1, min(n_full, target_s / max(one, 1e-6))))
        sig = np.float32(p.sigma_p2)
        for _ in range(k):
            sig = np.float32(sig * np.float32(p.sigma_factor))
        t0 = time.perf_counter()
        O.emicp(X, Y, sigma_p2=p.sigma_p2, sigma_inf=float(sig), sigma_factor=p.sigma_factor,
                d_02=p.d_02, precision="f32", trace=False)
        dt = time.perf_counter() - t0
    elif kind == "icp":
        t0 = time.perf_counter()
        O.icp(X, Y, maxIteration=1, precision="f32", trace=False)
        one = time.perf_counter() - t0
        k = int(max(1, min(n_full, target_s / max(one, 1e-6))))
        t0 = time.perf_counter()
        O.icp(X, Y, maxIteration=k, precision="f32", trace=False)
        dt = time.perf_counter() - t0
    else:
        t0 = time.perf_counter()
        O.softassign(X, Y, JMAX=1, I0=1, I1=p.I1, alpha=p.alpha, T_0=p.T_0, TFACTOR=p.TFACTOR,
                     moutlier=p.moutlier, precision="f32", trace=False)
        one = time.perf_counter() - t0
        k = int(max(1, min(n_full, target_s / max(one, 1e-6))))
        t0 = time.perf_counter()
        O.softassign(X, Y, JMAX=1, I0=k, I1=p.I1, alpha=p.alpha, T_0=p.T_0, TFACTOR=p.TFACTOR,
                     moutlier=p.moutlier, precision="f32", trace=False)
        dt = time.perf_counter() - t0
    per_update = dt / k
    regs_per_s = 1.0 / (per_update * n_full)
    desc = ("first %d of %d pose updates of one registration (FP32 port of the reference algorithm, "
            "OpenMP), scaled to a full registration" % (k, n_full))
    if kind == "icp":
        desc += "; ICP's port searches exhaustively (the reference's FLANN kd-tree is not available)"
    return regs_per_s, desc, threads


def run_reference(args, rank, world):
    if rank != 0:
        return
    if args.workload == BATCH_WORKLOAD:
        pairs = batch_workload(args.seed)
        per_step = max(0.5, args.cpu_sample_s / max(1, args.steps + args.warmup))
        vals = []
        for i in range(args.warmup + args.steps):
            v, desc, thr = batch_cpu_baseline(pairs, per_step)
            if i >= args.warmup:
                vals.append(v)
        value = float(np.mean(vals))
        line = {"impl": "reference", "metric": "registrations/s", "value": value, "unit": "registrations/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * len(pairs) / value,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": batch_config(args, pairs),
                "cpu_baseline": {"value": value, "unit": "registrations/s", "cores": thr, "kind": "port",
                                 "sample": desc},
                "e2e": {"value": value, "unit": "registrations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    kind, X, Y = workload(args.workload, args.seed)
    p = RefDefaults()
    per_step = max(0.5, args.cpu_sample_s / max(1, args.steps + args.warmup))
    vals = []
    for i in range(args.warmup + args.steps):
        v, desc, thr = cpu_baseline(kind, X, Y, p, per_step)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    line = {"impl": "reference", "metric": "registrations/s", "value": value, "unit": "registrations/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / value,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_of(args, kind, X, Y, p),
            "cpu_baseline": {"value": value, "unit": "registrations/s", "cores": thr, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "registrations/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(args, kind, X, Y, p):
    c = {"workload": args.workload, "algorithm": kind, "N": int(len(X)), "M": int(len(Y)),
         "pose_updates_per_registration": pose_updates(kind, p), "seed": args.seed,
         "l2": "flushed between steps (256 MiB write), outside the timed events",
         "parallelism": "replicas" if args.gpus > 1 else "single GPU"}
    if kind == "softassign":
        c.update(JMAX=p.JMAX, I0=p.I0, I1=p.I1, alpha=p.alpha, T_0=p.T_0, TFACTOR=p.TFACTOR)
    elif kind == "icp":
        c.update(maxIteration=p.maxIteration, search="exhaustive nearest neighbour")
    else:
        c.update(sigma_p2=p.sigma_p2, sigma_inf=p.sigma_inf, sigma_factor=p.sigma_factor, d_02=p.d_02)
    return c


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


BATCH_WORKLOAD = "c4_batch_256"


def batch_workload(seed, count=256):
    """Config 4: 256 pairs, N and M log-uniform in [500, 20000], config-1
    generator per pair; even pairs EM-ICP (default parameters), odd pairs
    Softassign (config-2 parameters, JMAX = 60)."""
    import cuda_emicp_softassign_gb300 as cesa
    from cuda_emicp_softassign_gb300 import workloads as W
    out = []
    for kind, X, Y, _, _ in W.batch_pairs(count=count, seed=seed):
        if kind == "emicp":
            out.append((cesa.ALGO_EMICP, X, Y, cesa.Params.default()))
        else:
            out.append((cesa.ALGO_SOFTASSIGN, X, Y, cesa.Params.default(JMAX=60)))
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
    return {"workload": BATCH_WORKLOAD, "pairs": len(pairs),
            "emicp_pairs": sum(1 for a, _, _, _ in pairs if a == 0),
            "softassign_pairs": sum(1 for a, _, _, _ in pairs if a == 1),
            "N_range": [int(min(n)), int(max(n))], "M_range": [int(min(m)), int(max(m))],
            "softassign_JMAX": 60, "seed": args.seed,
            "l2": "flushed between steps (256 MiB write), outside the timed events",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


def batch_cpu_baseline(pairs, target_s):
    """FP32 port of the reference algorithm on the host: time per affinity
    element measured on the first pose updates of a few pairs of the batch,
    scaled to the batch's total elements. Returns (registrations/s, desc, threads)."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    _, _, total = batch_work(pairs)
    spent = 0.0
    elems = 0.0
    used = 0
    for algo, X, Y, p in pairs[:8]:
        if spent > target_s:
            break
        t0 = time.perf_counter()
        if algo == 0:
            O.emicp(X, Y, sigma_p2=p.sigma_p2, sigma_inf=p.sigma_p2 * 0.5, sigma_factor=p.sigma_factor,
                    d_02=p.d_02, precision="f32", trace=False)
            n = pose_updates("emicp", type("P", (), dict(sigma_p2=p.sigma_p2, sigma_inf=p.sigma_p2 * 0.5,
                                                          sigma_factor=p.sigma_factor))())
            elems += float(len(X)) * len(Y) * n
        else:
            O.softassign(X, Y, JMAX=1, I0=1, I1=p.I1, alpha=p.alpha, T_0=p.T_0, TFACTOR=p.TFACTOR,
                         moutlier=p.moutlier, precision="f32", trace=False)
            elems += float(len(X)) * len(Y) * (2 * p.I1 + 1)
        spent += time.perf_counter() - t0
        used += 1
    per_elem = spent / elems
    regs = len(pairs) / (per_elem * total)
    desc = ("first pose updates of %d of the %d pairs (FP32 port of the reference algorithm, OpenMP): "
            "%.3g s per affinity element, scaled to the batch's %.3g elements" % (used, len(pairs), per_elem, total))
    return regs, desc, threads


def run_batch(args, rank, world, local):
    """Config 4: one step = one batched registration of all 256 pairs
    (cesa_register_batch_device, inputs resident). Also reported: the same
    pairs registered one pair per launch with the single-pair kernels."""
    import torch
    import cuda_emicp_softassign_gb300 as cesa

    torch.cuda.set_device(local)
    pairs = batch_workload(args.seed)
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

    # the same pairs, one pair per launch (single-pair device entry points)
    single_ms = 0.0
    for algo, dX, dY, dRt, p in dev:
        dRt.copy_(pose0)
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        (cesa.emicp_device if algo == 0 else cesa.softassign_device)(dX, dY, dRt, param=p, d_status=status,
                                                                      stream=stream)
        e1.record(stream)
        e1.synchronize()
        single_ms += e0.elapsed_time(e1)

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
    cpu_v, cpu_desc, cpu_thr = batch_cpu_baseline(pairs, args.cpu_sample_s)
    h2d = sum((len(X) + len(Y)) * 3 * 4 + 48 for _, X, Y, _ in pairs)
    line = {"metric": "registrations/s", "value": value, "unit": "registrations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator of config 4; see cuda_emicp_softassign_gb300/workloads.py)",
            "config": batch_config(args, pairs),
            "gelem_per_s": elems * args.steps * world / (total_ms * 1e-3) / 1e9,
            "one_pair_per_launch": {"value": world * npairs / (single_ms * 1e-3), "unit": "registrations/s",
                                    "ms": single_ms, "batched_speedup": single_ms / (total_ms / args.steps)},
            "roofline": roofline,
            "cpu_baseline": {"value": cpu_v, "unit": "registrations/s", "cores": cpu_thr, "kind": "port",
                             "sample": cpu_desc},
            "e2e": {"value": world * npairs / e2e_s, "unit": "registrations/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 48 * npairs},
            "clocks": clocks,
            "gpu_launches": 3 * args.steps,
            "wall_s_timed_region": t_wall}
    print(json.dumps(line), flush=True)


def measure_adjoint(cesa, kind, dX, dY, N, M, p, pose0, reps=3):
    """Forward + adjoint (cesa_<kind>_forward_device then
    cesa_<kind>_backward_device for the loss |R - I|^2 + |t|^2), CUDA events.
    Returns the plain forward, taped forward and backward milliseconds (best of
    reps) and (taped forward + backward) / plain forward. Softassign's taped
    forward runs the matrix-free kernel, so its plain forward is timed in that
    form too."""
    import copy
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
        ("taped forward (matrix-free) records the input pose and slack s, u of every pose update; the backward "
         "recomputes each update's Sinkhorn scalings and affinities (no N x M storage)")
    return {"fwd_ms": best[0], "fwd_taped_ms": best[1], "bwd_ms": best[2],
            "fwd_plus_bwd_over_fwd": (best[1] + best[2]) / best[0], "tape_bytes": int(nbytes),
            "loss": "|R - I|_F^2 + |t|^2 of the registered pose", "note": note}


def run_ours(args, rank, world, local):
    import torch
    import torch.distributed as dist
    import cuda_emicp_softassign_gb300 as cesa

    torch.cuda.set_device(local)
    kind, X, Y = workload(args.workload, args.seed)
    p = params_for(cesa, kind, args.sinkhorn_form)
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

    def one_step():
        dRt.copy_(pose0)
        dev_call(dX, dY, dRt, param=p, d_status=status, stream=stream)

    for _ in range(args.warmup):
        flush.zero_()
        one_step()
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
    fp32_ops, ex2_ops, elems = algorithmic_work(kind, N, M, p)
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
                        "sequence (prep kernels included)"}
    form_used = None
    if kind == "softassign":
        # the form the library resolved for this request (AUTO: tuned or by size), as it reports it
        import copy
        q = copy.copy(p)
        q.JMAX = 1
        rep = cesa.softassign(X, Y, param=q, trace=True)[3]
        form_used = FORM_NAMES.get(rep.sinkhorn_form, str(rep.sinkhorn_form))
    if form_used == "banded":
        roofline["note"] += (". The banded form computes each affinity once per inner iteration and "
                             "keeps the tile in shared memory for the other 2*I1 sweeps, so it executes "
                             "fewer operations than this per-sweep count: per element and pose update 1 ex2 "
                             "and %d FP32 ops (the first row sweep 8, each later Sinkhorn sweep 1, the final "
                             "sweep 5)" % (8 + (2 * p.I1 - 1) + 5))
        roofline["kernel"] = "softassign_band_kernel"
        roofline["executed_fp32_ops_per_registration"] = float(N) * float(M) * pose_updates(kind, p) * (
            8 + (2 * p.I1 - 1) + 5)
    if form_used == "materialised":
        hbm_peak = None
        try:
            hbm_peak = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json")))["hbm_gbs"]
        except (OSError, KeyError, ValueError):
            pass
        gbs = materialised_bytes(N, M, p) / mean_s / 1e9
        roofline = {"bound": "hbm", "kernel": "softassign_mat_kernel", "achieved": gbs,
                    "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak if hbm_peak else None,
                    "traffic": None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)",
                    "bytes_per_registration": materialised_bytes(N, M, p),
                    "note": "achieved = algorithmic HBM bytes (4 B per element written once and read by "
                            "each of the 2*I1 later passes, per pose update) / event time"}
    traffic_file = os.path.join(HERE, "profiles", "ncu_traffic.json")
    if os.path.exists(traffic_file):
        key = args.workload + (":" + form_used if form_used in ("materialised", "banded") else "")
        entry = json.load(open(traffic_file)).get(key)
        if entry:
            roofline["traffic"] = entry["bytes_per_launch"]
            roofline["traffic_source"] = "ncu dram bytes per launch, profiles/ncu_traffic.json"
    cpu_v, cpu_desc, cpu_thr = cpu_baseline(kind, X, Y, p, args.cpu_sample_s)
    h2d = (N + M) * 3 * 4 + 12 * 4
    line = {"metric": "registrations/s", "value": value, "unit": "registrations/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator of the workload; see cuda_emicp_softassign_gb300/workloads.py)",
            "config": config_of(args, kind, X, Y, p),
            "gelem_per_s": elems * regs / (total_ms * 1e-3) / 1e9,
            "roofline": roofline,
            "cpu_baseline": {"value": cpu_v, "unit": "registrations/s", "cores": cpu_thr, "kind": "port",
                             "sample": cpu_desc},
            "e2e": {"value": whole_job_rate(args.steps, world, e2e_s), "unit": "registrations/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 12 * 4},
            "clocks": clocks,
            "gpu_launches": kernels_per_registration(kind, form_used) * args.steps,
            "wall_s_timed_region": t_wall}
    if kind == "softassign":
        line["config"]["sinkhorn_form"] = form_used
        line["config"]["sinkhorn_tuner"] = tuned
    if kind == "icp":
        # value is the default search (a uniform grid from 4096 target points on), whose work depends
        # on the data; the FP32 roofline is that of the exhaustive search, timed here on the same pair
        import copy
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
        line["icp_search"] = {"value_search": "grid" if N >= 4096 else "exhaustive",
                              "ms_per_step": total_ms / args.steps, "exhaustive_ms_per_step": exh_s * 1e3,
                              "note": "both searches are exact and return the same matches"}
    if not args.no_adjoint and kind != "icp":
        adj = measure_adjoint(cesa, kind, dX, dY, N, M, p, pose0)
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
