// Batched registration for sm_103a: many (X, Y) pairs of uneven sizes, EM-ICP
// and Softassign mixed, in one persistent cooperative launch.
//
// Every pair follows its own schedule (the sigma loop of src/emicp.cu:443-669
// or the JMAX x I0 x I1 loops of src/softassign.cu:486-822), and all pairs
// advance in lock step, one phase per round:
//   EM-ICP      E (E-step sweep)  Z (moments -> S -> Horn pose)
//   Softassign  R_0 C_0 ... R_{I1-1} C_{I1-1} F Z
// with R_k / C_k the Sinkhorn row / column passes and F the final sweep. A
// sweep phase is split into (pair, tile) units of 128 owned points x one slice
// of the streamed points; a Z phase is one unit. The units of all pairs in a
// round form one work list, taken round-robin by the blocks of the grid, and
// the round ends at a grid barrier. With hundreds of pairs a round holds
// thousands of units, so the barrier is amortised and the small pairs (which
// alone could not fill 152 SMs) run alongside the large ones.
//
// Completion is by arrival counter: the last unit of an owned block sums the
// slice partials in slice order and completes the block (new Sinkhorn scaling
// and slack, or the block's moment record). The Z unit of a pair reduces the
// block records in a fixed order. Results therefore do not depend on which
// block ran which unit. The element functors, row finalizers and moment
// assembly are those of the single-pair kernels; the single-pair Softassign
// kernel completes its Sinkhorn passes differently (in the next pass), so the
// two agree to rounding, not bit for bit.
#include <cuda_runtime.h>

#include <vector>

#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {
namespace {

constexpr int kPhIdle = 0, kPhEmE = 1, kPhEmZ = 2, kPhSaRow = 3, kPhSaCol = 4, kPhSaFin = 5, kPhSaZ = 6;

// Per-pair state block (floats): [0..8] R, [9..11] t' (centred frame),
// [12] sigma_p2 (EM-ICP) or T (Softassign), [16..35] Horn eigenbasis and
// last quaternion.
constexpr int kStateFloats = 64;
constexpr int kStateHorn = 16;
static_assert(sizeof(HornState<float>) == 20 * sizeof(float), "Horn state layout");

// Streamed points per unit slice (two TMA chunks).
constexpr int kBatchSlice = 2 * kChunk;

struct BPair {
  int algo;  // 0 EM-ICP, 1 Softassign
  int N, M;
  SweepGeom g0;  // EM-ICP: own Y' stream X'; Softassign row sweeps: own X' stream Y'
  SweepGeom g1;  // Softassign column sweeps: own Y' stream X'
  int rounds;
  int nsteps;  // sigma steps or pose updates (JMAX * I0)
  int I0, I1;
  float init;  // sigma_p2 or T_0
  float sigma_factor, d_02;
  float alpha, TFACTOR, moutlier;
  const float* X;  // caller SoA (device)
  const float* Y;
  float* dRt;  // caller pose (device), written after the last step
  float4* own0;  // EM-ICP: Y' (M); Softassign: X' (N)
  float4* own1;  // EM-ICP: X' (N); Softassign: Y' (M)
  CenterHdr* hdr;
  float* part;
  unsigned* cnt0;
  unsigned* cnt1;
  df* rec;  // block moment records
  float *a, *s, *rs;  // Softassign rows [N]
  float *b, *u, *cs;  // Softassign columns [M]
  float* state;
};

struct BatchArgs {
  const BPair* pairs;
  int npairs;
  int rounds;  // max over pairs
  Ctl* ctl;
  int* d_status;
  uint64_t timeout_ns;
};

struct Sched {
  int algo, rounds, I1, units0, units1;
};

struct Ph {
  int phase, k, step;
  unsigned geo_round;  // sweeps of this geometry the pair has completed before
};

__device__ __forceinline__ Ph phase_of(const Sched& s, int r) {
  Ph p{kPhIdle, 0, 0, 0u};
  if (r >= s.rounds) return p;
  if (s.algo == 0) {
    p.step = r >> 1;
    p.phase = (r & 1) ? kPhEmZ : kPhEmE;
    p.geo_round = (unsigned)p.step;
    return p;
  }
  const int per = 2 * s.I1 + 2;
  const int upd = r / per, k = r - upd * per;
  p.step = upd;
  if (k < 2 * s.I1) {
    p.k = k >> 1;
    if (k & 1) {
      p.phase = kPhSaCol;
      p.geo_round = (unsigned)(upd * s.I1 + p.k);
    } else {
      p.phase = kPhSaRow;
      p.geo_round = (unsigned)(upd * (s.I1 + 1) + p.k);
    }
  } else if (k == 2 * s.I1) {
    p.phase = kPhSaFin;
    p.geo_round = (unsigned)(upd * (s.I1 + 1) + s.I1);
  } else {
    p.phase = kPhSaZ;
  }
  return p;
}

__device__ __forceinline__ int phase_units(const Sched& s, int phase) {
  switch (phase) {
    case kPhEmE:
    case kPhSaRow:
    case kPhSaFin:
      return s.units0;
    case kPhSaCol:
      return s.units1;
    case kPhEmZ:
    case kPhSaZ:
      return 1;
    default:
      return 0;
  }
}

// Exclusive prefix over the pairs of the units each has in round r
// (pref[npairs] = total). Block-wide.
__device__ void round_prefix(const Sched* sched, int npairs, int r, int* pref) {
  __shared__ int s_wsum[kWarps];
  const int per = (npairs + kThreads - 1) / kThreads;
  const int lo = min((int)threadIdx.x * per, npairs), hi = min(lo + per, npairs);
  int local = 0;
  for (int p = lo; p < hi; ++p) local += phase_units(sched[p], phase_of(sched[p], r).phase);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int v = local;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, v, off);
    if (lane >= off) v += n;
  }
  if (lane == 31) s_wsum[warp] = v;
  __syncthreads();
  int excl = v - local;
  for (int w = 0; w < warp; ++w) excl += s_wsum[w];
  for (int p = lo; p < hi; ++p) {
    pref[p] = excl;
    excl += phase_units(sched[p], phase_of(sched[p], r).phase);
  }
  if (threadIdx.x == kThreads - 1) pref[npairs] = excl;
  __syncthreads();
}

// Pair owning unit u of the round: the first p with pref[p + 1] > u.
__device__ __forceinline__ int pair_of_unit(const int* pref, int npairs, int u) {
  int lo = 0, hi = npairs;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (pref[mid + 1] <= u) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

struct UnitRef {
  int p;
  Ph ph;
  int blk, sl;
  SweepGeom g;
  const float4* src;  // streamed points (nullptr for a Z unit)
};

struct Task {
  const float4* src;  // nullptr: none
  int first, len;
};

__device__ __forceinline__ UnitRef resolve(const BPair* pairs, const Sched* sched, const int* pref, int npairs,
                                           int r, int u) {
  UnitRef U;
  U.p = pair_of_unit(pref, npairs, u);
  U.ph = phase_of(sched[U.p], r);
  const int lu = u - pref[U.p];
  const BPair& P = pairs[U.p];
  U.g = (U.ph.phase == kPhSaCol) ? P.g1 : P.g0;
  U.blk = lu / U.g.slices;
  U.sl = lu - U.blk * U.g.slices;
  switch (U.ph.phase) {
    case kPhEmE:
    case kPhSaRow:
    case kPhSaFin:
      U.src = P.own1;
      break;
    case kPhSaCol:
      U.src = P.own0;
      break;
    default:
      U.src = nullptr;
  }
  return U;
}

__device__ __forceinline__ Task first_task(const UnitRef& U) {
  Task t{U.src, 0, 0};
  if (!U.src) return t;
  const int sb = U.sl * U.g.slice_len;
  const int se = min(sb + U.g.slice_len, U.g.n_stream);
  t.first = sb;
  t.len = min(kChunk, se - sb);
  return t;
}

// Two-stage ring of TMA destinations; copies alternate between the stages.
struct Ring {
  unsigned uses[kStages];
  int next;
};

struct Slot {
  int stage;
  unsigned par;
  bool valid;
};

__device__ __forceinline__ Slot ring_issue(Ring& rg, SweepSmem& sm, const Task& t) {
  Slot s{rg.next, 0u, true};
  rg.next ^= 1;
  rg.uses[s.stage] += 1;
  s.par = (rg.uses[s.stage] - 1u) & 1u;
  if (threadIdx.x == 0) {
    const unsigned bytes = (unsigned)t.len * 16u;
    mbar_arrive_expect_tx(&sm.full[s.stage], bytes);
    bulk_g2s(&sm.raw[s.stage][0], t.src + t.first, bytes, &sm.full[s.stage]);
  }
  return s;
}

// One sweep unit: owned points (optionally posed), the slice streamed through
// the ring chunk by chunk, then split completion. The unit's first chunk is in
// `cur`; during its last chunk the first chunk of the block's next unit (`tn`)
// is issued into `nslot`.
template <int NACC, class Elem, class Prep, class Fin>
__device__ bool run_sweep_unit(SweepSmem& sm, Ring& rg, const UnitRef& U, const float4* own, bool xform,
                               const float (&R)[9], const float (&tc)[3], Slot cur, const Task& tn, Slot& nslot,
                               float* part, unsigned* cnt, const Elem& elem, const Prep& prep, const Fin& fin,
                               Ctl* ctl, uint64_t timeout_ns, int where) {
  const int warp = threadIdx.x >> 5;
  const SweepGeom& g = U.g;
  float4 ow[kOwnPerLane];
  bool valid[kOwnPerLane];
  load_owned(own, g.n_own, U.blk, ow, valid);
  float p[kOwnPerLane][3];
#pragma unroll
  for (int j = 0; j < kOwnPerLane; ++j) {
    if (xform) {
      p[j][0] = R[0] * ow[j].x + R[1] * ow[j].y + R[2] * ow[j].z + tc[0];
      p[j][1] = R[3] * ow[j].x + R[4] * ow[j].y + R[5] * ow[j].z + tc[1];
      p[j][2] = R[6] * ow[j].x + R[7] * ow[j].y + R[8] * ow[j].z + tc[2];
    } else {
      p[j][0] = ow[j].x;
      p[j][1] = ow[j].y;
      p[j][2] = ow[j].z;
    }
  }
  float acc[kOwnPerLane][NACC];
#pragma unroll
  for (int j = 0; j < kOwnPerLane; ++j)
#pragma unroll
    for (int a = 0; a < NACC; ++a) acc[j][a] = 0.f;
  nslot.valid = false;
  const int sb = U.sl * g.slice_len, se = min(sb + g.slice_len, g.n_stream);
  for (int first = sb; first < se; first += kChunk) {
    const int len = min(kChunk, se - first);
    Slot nx{0, 0u, false};
    if (first + kChunk < se) {
      nx = ring_issue(rg, sm, Task{U.src, first + kChunk, min(kChunk, se - first - kChunk)});
    } else if (tn.src) {
      nslot = ring_issue(rg, sm, tn);
    }
    const bool bad = !mbar_wait(&sm.full[cur.stage], cur.par, ctl, timeout_ns, where);
    if (__syncthreads_or(bad)) {  // leave only after the copies issued above have landed
      if (nx.valid) mbar_wait(&sm.full[nx.stage], nx.par, ctl, timeout_ns, where + 1);
      if (nslot.valid) mbar_wait(&sm.full[nslot.stage], nslot.par, ctl, timeout_ns, where + 1);
      nslot.valid = false;
      return false;
    }
    const PrepOut pb = prep(sm, cur.stage, first, len, U.blk);
    const float4* __restrict__ bufA = pb.a;
    const float4* __restrict__ bufB = pb.b;
#pragma unroll 2
    for (int c = warp; c < len; c += kWarps) {
      const float4 a = bufA[c];
      const float4 b = bufB[c];
#pragma unroll
      for (int j = 0; j < kOwnPerLane; ++j) elem(acc[j], p[j], a, b);
    }
    __syncthreads();
    cur = nx;
  }
  float tot[NACC];
  reduce_warps<NACC>(sm, acc, tot);
  if (split_complete<NACC>(sm, g, U.blk, U.sl, U.ph.geo_round, part, cnt, tot)) fin(U.blk, tot);
  return true;
}

// ---------------------------------------------------------------- Softassign
// Streamed Y' for a row pass: (R y' + t', b_c), b = 1 in the first pass of a
// pose update.
struct BRowPrep {
  float R[9], tc[3];
  const float* b;  // nullptr: 1
  __device__ __forceinline__ PrepOut operator()(SweepSmem& sm, int stage, int first, int len, int) const {
    for (int c = threadIdx.x; c < len; c += kThreads) {
      const float4 y = sm.raw[stage][c];
      const float w = b ? __ldcg(b + first + c) : 1.f;
      sm.prep[c] = make_float4(R[0] * y.x + R[1] * y.y + R[2] * y.z + tc[0],
                               R[3] * y.x + R[4] * y.y + R[5] * y.z + tc[1],
                               R[6] * y.x + R[7] * y.y + R[8] * y.z + tc[2], w);
    }
    __syncthreads();
    return PrepOut{sm.prep, sm.raw2[stage]};
  }
};

// Streamed X' for a column pass: (x', a_r) with a from the completed row pass.
struct BColPrep {
  const float* a;
  __device__ __forceinline__ PrepOut operator()(SweepSmem& sm, int stage, int first, int len, int) const {
    for (int c = threadIdx.x; c < len; c += kThreads) {
      const float4 x = sm.raw[stage][c];
      sm.prep[c] = make_float4(x.x, x.y, x.z, __ldcg(a + first + c));
    }
    __syncthreads();
    return PrepOut{sm.prep, sm.raw2[stage]};
  }
};

// Streamed Y' for the final sweep: (R y' + t', b) and (g (y' - Yhat), b (cs - 1))
// with g = b cs, from the completed last column pass.
struct BFinPrep {
  float R[9], tc[3], yh[3];
  const float* b;
  const float* cs;
  __device__ __forceinline__ PrepOut operator()(SweepSmem& sm, int stage, int first, int len, int) const {
    for (int c = threadIdx.x; c < len; c += kThreads) {
      const float4 y = sm.raw[stage][c];
      const float bn = __ldcg(b + first + c), csv = __ldcg(cs + first + c);
      const float g = bn * csv;
      sm.prep[c] = make_float4(R[0] * y.x + R[1] * y.y + R[2] * y.z + tc[0],
                               R[3] * y.x + R[4] * y.y + R[5] * y.z + tc[1],
                               R[6] * y.x + R[7] * y.y + R[8] * y.z + tc[2], bn);
      sm.prep2[c] = make_float4(g * (y.x - yh[0]), g * (y.y - yh[1]), g * (y.z - yh[2]), bn * (csv - 1.f));
    }
    __syncthreads();
    return PrepOut{sm.prep, sm.prep2};
  }
};

// Row pass completion (normalizeMbySinkhorn_row + Saxpy, src/softassign.cu:538-561):
//   rs = a_old (K b row sum) + s_old,  a = a_old / rs,  s = s_old / rs.
struct BRowFin {
  float *a, *s, *rs;
  int N;
  bool first;  // a_old = 1
  __device__ __forceinline__ void operator()(int blk, const float (&tot)[1]) const {
    const int r = blk * kBlockPts + (int)threadIdx.x;
    if (threadIdx.x < kBlockPts && r < N) {
      const float ao = first ? 1.f : __ldcg(a + r);
      const float so = __ldcg(s + r);
      const float rsv = fmaf(ao, tot[0], so);
      __stcg(a + r, ao / rsv);
      __stcg(s + r, so / rsv);
      __stcg(rs + r, rsv);
    }
  }
};

// Column pass completion (normalizeMbySinkhorn_col + Saxpy, src/softassign.cu:579-597):
//   cs = b_old (K^T a column sum) + u_old,  b = b_old / cs,  u = u_old / cs.
// After the last column pass of a pose update the block also stores its
// column moments sum cs and sum cs y' (record slots 28..31).
struct BColFin {
  float *b, *u, *cs;
  int M;
  bool first;    // b_old = 1
  bool moments;  // last column pass
  const float4* cols;
  df* scratch;  // shared, >= 33 * 128 dfs
  df* rec;      // column-block records [nblk1][32]
  __device__ __forceinline__ void operator()(int blk, const float (&tot)[1]) const {
    const int c = blk * kBlockPts + (int)threadIdx.x;
    float csv = 0.f;
    float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool mine = threadIdx.x < kBlockPts && c < M;
    if (mine) {
      const float bo = first ? 1.f : __ldcg(b + c);
      const float uo = __ldcg(u + c);
      csv = fmaf(bo, tot[0], uo);
      __stcg(b + c, bo / csv);
      __stcg(u + c, uo / csv);
      __stcg(cs + c, csv);
      if (moments) y = __ldcg(cols + c);
    }
    if (!moments) return;  // uniform
    df v[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = df_make(0.f);
    if (mine) {
      df_add(v[28], csv);
      df_add_prod(v[29], csv, y.x);
      df_add_prod(v[30], csv, y.y);
      df_add_prod(v[31], csv, y.z);
    }
    owned_block_sum<32>(v, scratch, rec + (size_t)blk * 32);
  }
};

// ---------------------------------------------------------------- pose tasks
__device__ __forceinline__ void load_pose(const float* state, float* s_pose) {
  if (threadIdx.x < 12) s_pose[threadIdx.x] = __ldcg(state + threadIdx.x);
  __syncthreads();
}

// Horn solve + pose store by thread 0; the carried eigenbasis lives in the
// pair's state block between solves.
__device__ void horn_update(const BPair& P, const float S[9], const float Xcp[3], const float Yd[3], int step,
                            bool last) {
  HornState<float> st;
  float* sv = reinterpret_cast<float*>(&st);
  for (int k = 0; k < 20; ++k) sv[k] = __ldcg(P.state + kStateHorn + k);
  float q[4], gap = 0.f, lmax = 0.f, Rn[9], tn[3];
  horn_quaternion<float>(S, st, q, &gap, &lmax);
  quat_to_pose<float>(q, Xcp, Yd, Rn, tn);
  for (int k = 0; k < 20; ++k) __stcg(P.state + kStateHorn + k, sv[k]);
  for (int k = 0; k < 9; ++k) __stcg(P.state + k, Rn[k]);
  for (int k = 0; k < 3; ++k) __stcg(P.state + 9 + k, tn[k]);
  if (last) {
    float t[3];
    pose_from_centred(Rn, tn, P.hdr->oX, P.hdr->oY, t);
    for (int k = 0; k < 9; ++k) P.dRt[k] = Rn[k];
    for (int k = 0; k < 3; ++k) P.dRt[9 + k] = t[k];
  }
  (void)step;
}

__device__ void em_finalize(const BPair& P, const Ph& ph, df* s_red, df* s_tot) {
  reduce_block_partials<kEmNV>(P.rec, P.g0.nblk, s_red, s_tot);
  if (threadIdx.x == 0) {
    float Xc[3], Yc[3], S[9];
    em_moments_to_S(s_tot, Xc, Yc, S);
    horn_update(P, S, Xc, Yc, ph.step, ph.step + 1 == P.nsteps);
    __stcg(P.state + 12, __ldcg(P.state + 12) * P.sigma_factor);  // FP32, src/emicp.cu:668
  }
  __syncthreads();
}

__device__ void sa_finalize(const BPair& P, const Ph& ph, df* s_red, df* s_tot, float* s_S, float* s_v) {
  reduce_block_partials<kSaNV>(P.rec, P.g0.nblk + P.g1.nblk, s_red, s_tot);
  if (threadIdx.x < 12) {
    const CenterHdr* h = P.hdr;
    sa_moments_to_S(threadIdx.x, s_tot, h->oX, h->oY, h->ymean, s_S, s_v, s_v + 3, s_v + 6, s_v + 9);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float S[9], Xcp[3], Yd[3];
    for (int k = 0; k < 9; ++k) S[k] = s_S[k];
    for (int i = 0; i < 3; ++i) {
      Xcp[i] = s_v[i];
      Yd[i] = s_v[3 + i];
    }
    horn_update(P, S, Xcp, Yd, ph.step, ph.step + 1 == P.nsteps);
    if ((ph.step + 1) % P.I0 == 0)
      __stcg(P.state + 12, __ldcg(P.state + 12) * P.TFACTOR);  // FP32, src/softassign.cu:820
  }
  __syncthreads();
}

// ---------------------------------------------------------------- the kernel
__global__ void __launch_bounds__(kThreads, 2) batch_kernel(const BatchArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SweepSmem& sm = *reinterpret_cast<SweepSmem*>(smem_raw);
  Sched* s_sched = reinterpret_cast<Sched*>(smem_raw + sizeof(SweepSmem));
  int* s_pref = reinterpret_cast<int*>(s_sched + A.npairs);
  __shared__ float s_pose[12];
  __shared__ df s_red[kThreads];
  __shared__ df s_tot[kSaNV];
  __shared__ float s_S[9], s_v[12];

  const int tid = threadIdx.x;
  const int G = (int)gridDim.x;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&sm.full[s], 1);
    mbar_init_fence();
  }
  for (int p = tid; p < A.npairs; p += kThreads) {
    const BPair& P = A.pairs[p];
    s_sched[p] = Sched{P.algo, P.rounds, P.I1, P.g0.units, P.g1.units};
  }
  __syncthreads();

  Ring rg{{0u, 0u}, 0};
  unsigned epoch = 0;
  bool ok = true;
  for (int r = 0; r < A.rounds && ok; ++r) {
    round_prefix(s_sched, A.npairs, r, s_pref);
    const int total = s_pref[A.npairs];
    int u = blockIdx.x;
    if (u < total) {
      UnitRef cur = resolve(A.pairs, s_sched, s_pref, A.npairs, r, u);
      Slot slot{0, 0u, false};
      const Task t0 = first_task(cur);
      if (t0.src) slot = ring_issue(rg, sm, t0);
      for (;;) {
        const int un = u + G;
        UnitRef nxt{};
        Task tn{nullptr, 0, 0};
        if (un < total) {
          nxt = resolve(A.pairs, s_sched, s_pref, A.npairs, r, un);
          tn = first_task(nxt);
        }
        const BPair& P = A.pairs[cur.p];
        Slot ns{0, 0u, false};
        if (cur.ph.phase == kPhEmZ || cur.ph.phase == kPhSaZ) {
          if (tn.src) ns = ring_issue(rg, sm, tn);  // lands while the pose is solved
          if (cur.ph.phase == kPhEmZ) em_finalize(P, cur.ph, s_red, s_tot);
          else sa_finalize(P, cur.ph, s_red, s_tot, s_S, s_v);
        } else {
          load_pose(P.state, s_pose);
          float R[9], tc[3];
#pragma unroll
          for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
#pragma unroll
          for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
          const float par = __ldcg(P.state + 12);  // sigma_p2 or T
          df* scratch = reinterpret_cast<df*>(sm.prep);
          if (cur.ph.phase == kPhEmE) {
            const EmicpElem elem{-kLog2e / (2.f * par)};
            const CenterHdr* h = P.hdr;
            const EmicpFin fin{P.own0, P.M, expf(-P.d_02 / par),  // src/emicp.cu:489
                               {h->xmean[0], h->xmean[1], h->xmean[2]}, nullptr,
                               {h->oX[0], h->oX[1], h->oX[2]}, scratch, P.rec};
            ok = run_sweep_unit<5>(sm, rg, cur, P.own0, true, R, tc, slot, tn, ns, P.part, P.cnt0, elem,
                                   NoPrep{}, fin, A.ctl, A.timeout_ns, 10);
          } else {
            // K = exp((alpha - d^2)/T) / sqrt(T) = 2^(c0 + nk d^2)
            const float kk = kLog2e / par;
            const float c0 = fmaf(P.alpha, kk, -0.5f * log2f(par));
            if (cur.ph.phase == kPhSaRow) {
              BRowPrep prep;
#pragma unroll
              for (int k = 0; k < 9; ++k) prep.R[k] = R[k];
#pragma unroll
              for (int k = 0; k < 3; ++k) prep.tc[k] = tc[k];
              prep.b = cur.ph.k == 0 ? nullptr : P.b;
              const BRowFin fin{P.a, P.s, P.rs, P.N, cur.ph.k == 0};
              ok = run_sweep_unit<1>(sm, rg, cur, P.own0, false, R, tc, slot, tn, ns, P.part, P.cnt0,
                                     SinkElem{-kk, c0}, prep, fin, A.ctl, A.timeout_ns, 30);
            } else if (cur.ph.phase == kPhSaCol) {
              const BColFin fin{P.b, P.u, P.cs, P.M, cur.ph.k == 0, cur.ph.k == P.I1 - 1, P.own1, scratch,
                                P.rec + (size_t)P.g0.nblk * 32};
              ok = run_sweep_unit<1>(sm, rg, cur, P.own1, true, R, tc, slot, tn, ns, P.part, P.cnt1,
                                     SinkElem{-kk, c0}, BColPrep{P.a}, fin, A.ctl, A.timeout_ns, 40);
            } else {
              BFinPrep prep;
#pragma unroll
              for (int k = 0; k < 9; ++k) prep.R[k] = R[k];
#pragma unroll
              for (int k = 0; k < 3; ++k) {
                prep.tc[k] = tc[k];
                prep.yh[k] = P.hdr->ymean[k];
              }
              prep.b = P.b;
              prep.cs = P.cs;
              static_assert(offsetof(SweepSmem, full) - offsetof(SweepSmem, prep) >=
                                32 * (kBlockPts + 8) * sizeof(df),
                            "moment scratch does not fit");
              const FinalFin fin{P.own0, P.a, nullptr, P.N, scratch, P.rec};
              ok = run_sweep_unit<5>(sm, rg, cur, P.own0, false, R, tc, slot, tn, ns, P.part, P.cnt0,
                                     FinalElem{-kk, c0}, prep, fin, A.ctl, A.timeout_ns, 50);
            }
          }
        }
        if (!ok || un >= total) break;
        u = un;
        cur = nxt;
        slot = ns;
      }
    }
    ok = ok && grid_sync(A.ctl, epoch, (unsigned)G, A.timeout_ns, 70);
  }
  if (blockIdx.x == 0 && tid == 0) {
    const int st = ld_status(A.ctl);
    if (A.d_status) *A.d_status = st;
    if (st == kStatusOk) A.ctl->steps_done = A.rounds;
  }
}

// Per-pair init: centred points, slack vectors, pose in the centred frame.
__global__ void __launch_bounds__(1024) batch_center_kernel(const BPair* pairs) {
  const BPair& P = pairs[blockIdx.x];
  center_block(P.X, P.N, P.Y, P.M, P.hdr);
}

__global__ void batch_pack_kernel(const BPair* pairs) {
  const BPair& P = pairs[blockIdx.y];
  const CenterHdr* h = P.hdr;
  float4* xo = P.algo == 0 ? P.own1 : P.own0;
  float4* yo = P.algo == 0 ? P.own0 : P.own1;
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.N; i += stride) {
    xo[i] = make_float4(__fsub_rn(P.X[i], h->oX[0]), __fsub_rn(P.X[P.N + i], h->oX[1]),
                        __fsub_rn(P.X[2 * P.N + i], h->oX[2]), 0.f);
    if (P.algo == 1) P.s[i] = P.moutlier;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.M; i += stride) {
    yo[i] = make_float4(__fsub_rn(P.Y[i], h->oY[0]), __fsub_rn(P.Y[P.M + i], h->oY[1]),
                        __fsub_rn(P.Y[2 * P.M + i], h->oY[2]), 0.f);
    if (P.algo == 1) P.u[i] = P.moutlier;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    float R[9], t[3], tc[3];
    for (int k = 0; k < 9; ++k) R[k] = P.dRt[k];
    for (int k = 0; k < 3; ++k) t[k] = P.dRt[9 + k];
    pose_to_centred(R, t, h->oX, h->oY, tc);
    for (int k = 0; k < 9; ++k) P.state[k] = R[k];
    for (int k = 0; k < 3; ++k) P.state[9 + k] = tc[k];
    P.state[12] = P.init;
    HornState<float> st;
    st.reset();
    const float* sv = reinterpret_cast<const float*>(&st);
    for (int k = 0; k < 20; ++k) P.state[kStateHorn + k] = sv[k];
  }
}

struct Carve {
  char* p;
  size_t off = 0;
  explicit Carve(void* base) : p(static_cast<char*>(base)) {}
  template <class T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* r = p ? reinterpret_cast<T*>(p + off) : nullptr;
    off += n * sizeof(T);
    return r;
  }
};

SweepGeom batch_geom(int n_own, int n_stream) {
  SweepGeom g;
  g.n_own = n_own;
  g.n_stream = n_stream;
  g.nblk = (n_own + kBlockPts - 1) / kBlockPts;
  int S = (n_stream + kBatchSlice - 1) / kBatchSlice;
  if (S < 1) S = 1;
  g.slice_len = (n_stream + S - 1) / S;
  g.slices = (n_stream + g.slice_len - 1) / g.slice_len;
  g.units = g.nblk * g.slices;
  return g;
}

// Lays out the workspace: control block, all split counters (cleared per
// launch), the pair table, then each pair's buffers. With base == nullptr
// only sizes are computed.
size_t carve_batch(void* base, const BatchLaunchPair* in, int npairs, std::vector<BPair>* out, Ctl** ctl,
                   size_t* zero_bytes, BPair** dpairs, int* rounds) {
  Carve c(base);
  *ctl = c.take<Ctl>(1);
  std::vector<BPair> v((size_t)npairs);
  size_t ncnt = 0;
  for (int i = 0; i < npairs; ++i) {
    const BatchLaunchPair& L = in[i];
    BPair& P = v[(size_t)i];
    P = BPair{};
    P.algo = L.algo;
    P.N = L.N;
    P.M = L.M;
    if (L.algo == 0) {
      P.g0 = batch_geom(L.M, L.N);
      P.g1 = SweepGeom{0, 0, 0, 1, 0, 0};
      P.nsteps = L.nsteps;
      P.rounds = 2 * L.nsteps;
      P.init = L.sigma_p2;
      P.sigma_factor = L.sigma_factor;
      P.d_02 = L.d_02;
      P.I0 = 1;
      P.I1 = 1;
    } else {
      P.g0 = batch_geom(L.N, L.M);
      P.g1 = batch_geom(L.M, L.N);
      P.nsteps = L.JMAX * L.I0;
      P.rounds = (2 * L.I1 + 2) * P.nsteps;
      P.init = L.T_0;
      P.alpha = L.alpha;
      P.TFACTOR = L.TFACTOR;
      P.moutlier = L.moutlier;
      P.I0 = L.I0;
      P.I1 = L.I1;
    }
    ncnt += (size_t)P.g0.nblk + (size_t)P.g1.nblk;
    P.X = L.dX;
    P.Y = L.dY;
    P.dRt = L.dRt;
  }
  unsigned* cnt = c.take<unsigned>(ncnt > 0 ? ncnt : 1);
  *zero_bytes = c.off;
  *dpairs = c.take<BPair>((size_t)npairs);
  int rmax = 0;
  size_t co = 0;
  for (int i = 0; i < npairs; ++i) {
    BPair& P = v[(size_t)i];
    const int n0 = P.algo == 0 ? P.M : P.N;
    const int n1 = P.algo == 0 ? P.N : P.M;
    P.cnt0 = cnt ? cnt + co : nullptr;
    co += (size_t)P.g0.nblk;
    P.cnt1 = cnt ? cnt + co : nullptr;
    co += (size_t)P.g1.nblk;
    P.hdr = c.take<CenterHdr>(1);
    P.own0 = c.take<float4>((size_t)n0);
    P.own1 = c.take<float4>((size_t)n1);
    const size_t part0 = (size_t)P.g0.units * 5 * kBlockPts;
    const size_t part1 = (size_t)P.g1.units * 1 * kBlockPts;
    P.part = c.take<float>(part0 > part1 ? part0 : part1);
    P.rec = c.take<df>((size_t)(P.g0.nblk + P.g1.nblk) * 32);
    if (P.algo == 1) {
      P.a = c.take<float>((size_t)P.N);
      P.s = c.take<float>((size_t)P.N);
      P.rs = c.take<float>((size_t)P.N);
      P.b = c.take<float>((size_t)P.M);
      P.u = c.take<float>((size_t)P.M);
      P.cs = c.take<float>((size_t)P.M);
    }
    P.state = c.take<float>(kStateFloats);
    if (P.rounds > rmax) rmax = P.rounds;
  }
  if (out) out->swap(v);
  *rounds = rmax;
  return c.off;
}

size_t batch_smem(int npairs) {
  return sizeof(SweepSmem) + sizeof(Sched) * (size_t)npairs + sizeof(int) * ((size_t)npairs + 1);
}

}  // namespace

size_t batch_ws_need(const BatchLaunchPair* pairs, int npairs) {
  Ctl* ctl = nullptr;
  size_t zb = 0;
  BPair* dp = nullptr;
  int rounds = 0;
  return carve_batch(nullptr, pairs, npairs, nullptr, &ctl, &zb, &dp, &rounds);
}

int enqueue_batch(const BatchLaunchPair* pairs, int npairs, int* d_status, uint64_t timeout_ns, void* ws,
                  size_t ws_bytes, cudaStream_t st, int* grid_used, int* rounds_out) {
  if (npairs < 1 || npairs > kMaxBatchPairs) return (int)cudaErrorInvalidValue;
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  std::vector<BPair> host;
  Ctl* ctl = nullptr;
  size_t zero_bytes = 0;
  BPair* dpairs = nullptr;
  int rounds = 0;
  const size_t need = carve_batch(ws, pairs, npairs, &host, &ctl, &zero_bytes, &dpairs, &rounds);
  if (need > ws_bytes) return (int)cudaErrorInvalidValue;
  if (rounds_out) *rounds_out = rounds;
  e = cudaMemsetAsync(ws, 0, zero_bytes, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dpairs, host.data(), sizeof(BPair) * (size_t)npairs, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return (int)e;
  batch_center_kernel<<<npairs, 1024, 0, st>>>(dpairs);
  batch_pack_kernel<<<dim3(16, npairs), 256, 0, st>>>(dpairs);
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  const size_t smem = batch_smem(npairs);
  const int limit = persistent_grid_limit(device, (const void*)batch_kernel, smem);
  if (grid_used) *grid_used = limit;
  if (rounds == 0) return 0;
  BatchArgs A;
  A.pairs = dpairs;
  A.npairs = npairs;
  A.rounds = rounds;
  A.ctl = ctl;
  A.d_status = d_status;
  A.timeout_ns = timeout_ns;
  void* args[] = {(void*)&A};
  e = cudaLaunchCooperativeKernel((const void*)batch_kernel, dim3(limit), dim3(kThreads), args, smem, st);
  return (int)e;
}

}  // namespace cesa
