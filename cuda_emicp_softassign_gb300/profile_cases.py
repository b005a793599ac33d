"""Small, fixed workloads for profiling single kernels (each runs its kernel
twice, so that a profiler can skip the first launch):

    python -m cuda_emicp_softassign_gb300.profile_cases <case>

cases:
  c2_one      softassign_band_kernel: one config-2 registration (N = M = 2000, default schedule,
              the form AUTO picks: banded)
  c2_one_mf   softassign_kernel: the same with the grid-wide matrix-free form
  c2_timeline softassign_band_kernel's in-kernel phase timeline on config 2 (JMAX = 4, 20 pose
              updates): prints the mean duration of each phase of a pose update in block 0 and the
              spread over blocks (no profiler; %globaltimer marks written by thread 0 of every block)
  c5_update   softassign_kernel: config 5 (N = M = 20000), matrix-free form, one pose update
  c3_short    emicp_kernel: config 3 (N = M = 40097) with sigma_inf = 2e-3 (first 16 sigma steps)
  batch_mid   batch_kernel: the first 64 config-4 pairs, EM-ICP to sigma_inf = 5e-3,
              Softassign with JMAX = 1, I0 = 2
  mat_8000    softassign_mat_kernel: N = M = 8000 (K is 258 MB), one pose update, materialised form
  adj_20000   emicp_adjoint_kernel: forward + backward, N = M = 20000, sigma_inf = 2e-3 (16 steps)
  sa_adj_20000  Softassign adjoint sweeps (k_sweep_sum, k_sweep_grad): forward + backward,
              N = M = 20000 (config-5 generator), JMAX = 1, I0 = 2 (two pose updates)
  icp_20000   icp_kernel: ICP on config 3's generator at N = M = 20000, 5 iterations, exhaustive search
  icp_grid_20000  icp_kernel: the same with the uniform-grid search
"""
import sys

import numpy as np


def c2_one():
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c2_softassign_2000", seed=0)
    for _ in range(2):
        C.softassign(X, Y)


def c2_one_mf():
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c2_softassign_2000", seed=0)
    p = C.Params.default(sinkhorn_form=C.SINKHORN_MATRIX_FREE)
    for _ in range(2):
        C.softassign(X, Y, param=p)


def c2_timeline():
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c2_softassign_2000", seed=0)
    p = C.Params.default(JMAX=4, sinkhorn_form=C.SINKHORN_BANDED)
    C.softassign(X, Y, param=p)
    _, _, tl, rep = C.softassign(X, Y, param=p, timeline=256 * 800)
    rows = C.timeline_table(tl, rep.grid_blocks)
    names = {1: "start", 2: "final: last column pass completed", 3: "row pass completed (cluster)",
             4: "column sweep + partial store (final: record store)",
             5: "barrier (column tile's CTAs; the grid before the pose)", 6: "moment records reduced",
             7: "Horn solve", 8: "cluster barrier (final sweep included after 2)", 10: "moments: cluster barrier",
             11: "final rows finalised", 12: "moments summed", 13: "S formed",
             14: "column pass completed (band partials)", 15: "row sweep + warp reduction"}
    b0 = rows[rows[:, 0] == 0][:, 1:]
    starts = np.where(b0[:, 0] == 1)[0]
    segs = [b0[a:b + 1] for a, b in zip(starts[1:-1], starts[2:])]
    print("form %d, grid %d, pose update (block 0, mean of %d): %.0f ns"
          % (rep.sinkhorn_form, rep.grid_blocks, len(segs), np.mean([s[-1, 1] - s[0, 1] for s in segs])))
    for i in range(1, len(segs[0])):
        d = np.mean([s[i, 1] - s[i - 1, 1] for s in segs])
        print("  %2d  %-42s %6.0f ns" % (i, names.get(int(segs[0][i, 0]), "next update"), d))


def c1_timeline():
    """Phases of a config-1 EM-ICP sigma step (block 0, mean over the steps)."""
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c1_emicp_1007", seed=0)
    C.emicp(X, Y)
    _, _, tl, rep = C.emicp(X, Y, timeline=304 * 4000)
    rows = C.timeline_table(tl, rep.grid_blocks)
    names = {1: "start", 2: "a unit's first chunk landed", 3: "unit swept", 4: "unit's row partials stored",
             5: "grid barrier after the sweep", 8: "rows completed, block moments, grid barrier",
             6: "moment records reduced", 7: "S (nine threads) + pose solve"}
    b0 = rows[rows[:, 0] == 0][:, 1:]
    starts = np.where(b0[:, 0] == 1)[0]
    segs = [b0[a:b + 1] for a, b in zip(starts[1:-1], starts[2:])]
    segs = [sg for sg in segs if len(sg) == len(segs[0])]
    print("grid %d, sigma step (block 0, mean of %d): %.0f ns"
          % (rep.grid_blocks, len(segs), np.mean([sg[-1, 1] - sg[0, 1] for sg in segs])))
    for i in range(1, len(segs[0])):
        d = np.mean([sg[i, 1] - sg[i - 1, 1] for sg in segs])
        print("  %2d  %-46s %6.0f ns" % (i, names.get(int(segs[0][i, 0]), "next step"), d))


def c2_horn():
    """The pose solve over a whole config-2 registration (banded form): how
    many updates the certified inverse iteration takes (the trace's gap is -1
    there) and the solve's duration per update from the timeline."""
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c2_softassign_2000", seed=0)
    p = C.Params.default(sinkhorn_form=C.SINKHORN_BANDED)
    _, _, tr, _ = C.softassign(X, Y, param=p, trace=True)
    fast = tr[:, 30] == -1
    print("pose updates %d, certified inverse iteration %d, Jacobi fallback at updates %s"
          % (len(fast), int(fast.sum()), np.where(~fast)[0].tolist()))
    _, _, tl, rep = C.softassign(X, Y, param=p, timeline=256 * 12000)
    b0 = C.timeline_table(tl, rep.grid_blocks)
    b0 = b0[b0[:, 0] == 0][:, 1:]
    i13 = np.where(b0[:-1, 0] == 13)[0]
    d = b0[i13 + 1, 1] - b0[i13, 1]
    print("solve (S formed -> pose), ns over %d updates: mean %.0f, median %.0f, p90 %.0f, max %.0f"
          % (len(d), d.mean(), np.median(d), np.percentile(d, 90), d.max()))


def c5_update():
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c5_softassign_20000", seed=0)
    p = C.Params.default(JMAX=1, I0=1, sinkhorn_form=C.SINKHORN_MATRIX_FREE)
    for _ in range(2):
        C.softassign(X, Y, param=p)


def c3_short():
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("c3_emicp_40097", seed=0)
    p = C.Params.default(sigma_inf=2e-3)
    for _ in range(2):
        C.emicp(X, Y, param=p)


def batch_mid():
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    args = []
    for kind, X, Y, _, _ in W.batch_pairs(count=64, seed=0):
        if kind == "emicp":
            args.append((C.ALGO_EMICP, X, Y, C.Params.default(sigma_inf=0.005)))
        else:
            args.append((C.ALGO_SOFTASSIGN, X, Y, C.Params.default(JMAX=1, I0=2)))
    for _ in range(2):
        C.register_batch(args)


def mat_8000():
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    X, Y, _, _ = W.surface_pair(n=8000, m=8000, seed=1)
    p = C.Params.default(JMAX=1, I0=1, sinkhorn_form=C.SINKHORN_MATERIALISED)
    for _ in range(2):
        C.softassign(X, Y, param=p)


def adj_20000():
    import torch

    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    from cuda_emicp_softassign_gb300.autograd import emicp_autograd
    _, X, Y, _, _ = W.make("c3_emicp_40097", seed=0, n=20000)
    p = C.Params.default(sigma_inf=2e-3)
    Xd = torch.tensor(np.asarray(X), dtype=torch.float32, device="cuda", requires_grad=True)
    Yd = torch.tensor(np.asarray(Y), dtype=torch.float32, device="cuda", requires_grad=True)
    R0 = torch.eye(3, device="cuda", requires_grad=True)
    t0 = torch.zeros(3, device="cuda", requires_grad=True)
    for _ in range(2):
        R, t = emicp_autograd(Xd, Yd, R0, t0, p)
        (R.sum() + t.sum()).backward()
    torch.cuda.synchronize()


def sa_adj_20000():
    import torch

    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    from cuda_emicp_softassign_gb300.autograd import softassign_autograd
    _, X, Y, _, _ = W.make("c5_softassign_20000", seed=0)
    p = C.Params.default(JMAX=1, I0=2)
    Xd = torch.tensor(np.asarray(X), dtype=torch.float32, device="cuda", requires_grad=True)
    Yd = torch.tensor(np.asarray(Y), dtype=torch.float32, device="cuda", requires_grad=True)
    R0 = torch.eye(3, device="cuda", requires_grad=True)
    t0 = torch.zeros(3, device="cuda", requires_grad=True)
    for _ in range(2):
        R, t = softassign_autograd(Xd, Yd, R0, t0, p)
        (R.sum() + t.sum()).backward()
    torch.cuda.synchronize()


def _icp(search):
    import cuda_emicp_softassign_gb300 as C
    from cuda_emicp_softassign_gb300 import workloads as W
    _, X, Y, _, _ = W.make("icp_40097", seed=0, n=20000)
    p = C.Params.default(maxIteration=5, icp_search=search)
    for _ in range(2):
        C.icp(X, Y, param=p)


def icp_20000():
    _icp(1)  # CESA_ICP_SEARCH_EXHAUSTIVE


def icp_grid_20000():
    _icp(2)  # CESA_ICP_SEARCH_GRID


CASES = {f.__name__: f for f in (c1_timeline, c2_one, c2_one_mf, c2_timeline, c2_horn, c5_update, c3_short, batch_mid, mat_8000, adj_20000, sa_adj_20000, icp_20000,
                                  icp_grid_20000)}

if __name__ == "__main__":
    if len(sys.argv) != 2 or sys.argv[1] not in CASES:
        sys.exit("usage: python -m cuda_emicp_softassign_gb300.profile_cases {%s}" % "|".join(CASES))
    CASES[sys.argv[1]]()
