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

#include <algorithm>
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

// Streamed points per unit slice: from one to kMaxSliceChunks TMA chunks,
// chosen so that a round holds about kUnitsPerBlock units per block.
constexpr int kMaxSliceChunks = 8;
constexpr double kUnitsPerBlock = 8.0;

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
  unsigned* rctr;  // [rounds] units handed out beyond the first G of each round
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

// Where a unit's data lands in the stage buffers: streamed points in
// raw[stage]; in raw2[stage] the streamed points' weights (floats [0, 512) and
// [512, 1024)) and, with a unit's first chunk, its owned points (float4
// [256, 384)).
constexpr int kOwnSlot = 256;
// With a unit's first chunk also the pair's state block (pose, sigma_p2 or T:
// 16 floats) and centring header (16 floats), at float4 [384, 392).
constexpr int kMetaSlot = kOwnSlot + kBlockPts;
static_assert(kOwnSlot * 4 >= 2 * kChunk && kMetaSlot + 8 <= kChunk, "stage buffer layout");
static_assert(sizeof(CenterHdr) == 16 * sizeof(float), "centring header layout");

struct UnitRef {
  int p;
  Ph ph;
  int blk, sl;
  SweepGeom g;
  const float4* src;  // streamed points (nullptr for a Z unit)
  const float4* own;  // owned points of the pair (all blocks)
  const float* w0;    // weights of the streamed points, or nullptr
  const float* w1;
  const float* state;  // the pair's state block
  const CenterHdr* hdr;
};

struct Task {
  const float4* src;  // nullptr: none
  int first, len;
  const float* w0;
  const float* w1;
  const float4* own;  // first chunk of a unit: its owned points, else nullptr
  int own_n;
  const float* state;  // first chunk: the pair's state block and centring header
  const CenterHdr* hdr;
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
  U.w0 = nullptr;
  U.w1 = nullptr;
  U.state = P.state;
  U.hdr = P.hdr;
  switch (U.ph.phase) {
    case kPhEmE:
      U.src = P.own1;
      U.own = P.own0;
      break;
    case kPhSaRow:
      U.src = P.own1;
      U.own = P.own0;
      U.w0 = U.ph.k == 0 ? nullptr : P.b;
      break;
    case kPhSaFin:
      U.src = P.own1;
      U.own = P.own0;
      U.w0 = P.b;
      U.w1 = P.cs;
      break;
    case kPhSaCol:
      U.src = P.own0;
      U.own = P.own1;
      U.w0 = P.a;
      break;
    default:
      U.src = nullptr;
      U.own = nullptr;
  }
  return U;
}

// The unit's chunk starting at `first` (the first chunk also carries the
// owned points).
__device__ __forceinline__ Task chunk_task(const UnitRef& U, int first, bool with_own) {
  Task t{U.src, first, 0, U.w0, U.w1, nullptr, 0, nullptr, nullptr};
  const int se = min(U.sl * U.g.slice_len + U.g.slice_len, U.g.n_stream);
  t.len = min(kChunk, se - first);
  if (with_own) {
    t.own = U.own + (size_t)U.blk * kBlockPts;
    t.own_n = min(kBlockPts, U.g.n_own - U.blk * kBlockPts);
    t.state = U.state;
    t.hdr = U.hdr;
  }
  return t;
}

__device__ __forceinline__ Task first_task(const UnitRef& U) {
  if (!U.src) return Task{nullptr, 0, 0, nullptr, nullptr, nullptr, 0, nullptr, nullptr};
  return chunk_task(U, U.sl * U.g.slice_len, true);
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

// Issues the bulk copies of one task on the next stage's mbarrier. Weight
// copies are rounded up to 4 floats (16 bytes): slices start at multiples of
// 4 points and the weight arrays are padded to a multiple of 4.
__device__ __forceinline__ Slot ring_issue(Ring& rg, SweepSmem& sm, const Task& t) {
  Slot s{rg.next, 0u, true};
  rg.next ^= 1;
  rg.uses[s.stage] += 1;
  s.par = (rg.uses[s.stage] - 1u) & 1u;
  if (threadIdx.x == 0) {
    const unsigned pbytes = (unsigned)t.len * 16u;
    const unsigned wbytes = (unsigned)((t.len + 3) & ~3) * 4u;
    const unsigned obytes = (unsigned)t.own_n * 16u;
    const unsigned total = pbytes + (t.w0 ? wbytes : 0u) + (t.w1 ? wbytes : 0u) + (t.own ? obytes : 0u) +
                           (t.state ? 128u : 0u);
    mbar_arrive_expect_tx(&sm.full[s.stage], total);
    bulk_g2s(&sm.raw[s.stage][0], t.src + t.first, pbytes, &sm.full[s.stage]);
    float* wd = reinterpret_cast<float*>(&sm.raw2[s.stage][0]);
    if (t.w0) bulk_g2s(wd, t.w0 + t.first, wbytes, &sm.full[s.stage]);
    if (t.w1) bulk_g2s(wd + kChunk, t.w1 + t.first, wbytes, &sm.full[s.stage]);
    if (t.own) bulk_g2s(&sm.raw2[s.stage][kOwnSlot], t.own, obytes, &sm.full[s.stage]);
    if (t.state) {
      bulk_g2s(&sm.raw2[s.stage][kMetaSlot], t.state, 64u, &sm.full[s.stage]);
      bulk_g2s(&sm.raw2[s.stage][kMetaSlot + 4], t.hdr, 64u, &sm.full[s.stage]);
    }
  }
  return s;
}

// One sweep unit: owned points (optionally posed), the slice streamed through
// the ring chunk by chunk, then split completion. The unit's first chunk
// brings its owned points and the pair's state and centring header (copied to
// `meta`: 16 state floats, then the header). `Ops` supplies the element
// constants, the prepare step (reading the pose from meta) and the finalize
// step. During the unit's last chunk the first chunk of the block's next unit
// (`tn`) is issued into `nslot`.
template <int NACC, class Ops>
__device__ bool run_sweep_unit(SweepSmem& sm, Ring& rg, const UnitRef& U, bool xform, Slot cur, const Task& tn,
                               Slot& nslot, float* part, unsigned* cnt, const Ops& ops, float* meta, Ctl* ctl,
                               uint64_t timeout_ns, int where) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const SweepGeom& g = U.g;
  typename Ops::Elem elem;
  float2 q[kPairs][3];
  float2 acc[kPairs][NACC];
#pragma unroll
  for (int k = 0; k < kPairs; ++k)
#pragma unroll
    for (int a = 0; a < NACC; ++a) acc[k][a] = make_float2(0.f, 0.f);
  nslot.valid = false;
  const int sb = U.sl * g.slice_len, se = min(sb + g.slice_len, g.n_stream);
  for (int first = sb; first < se; first += kChunk) {
    const int len = min(kChunk, se - first);
    Slot nx{0, 0u, false};
    if (first + kChunk < se) {
      nx = ring_issue(rg, sm, chunk_task(U, first + kChunk, false));
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
    if (first == sb) {  // owned points, state and header arrived with the first chunk
      const float* m = reinterpret_cast<const float*>(&sm.raw2[cur.stage][kMetaSlot]);
      if (threadIdx.x < 32) meta[threadIdx.x] = m[threadIdx.x];
      elem = ops.elem(m);
      const float sc = ops.scale(m);  // the phase's coordinate scale (both clouds)
      const float4* os = &sm.raw2[cur.stage][kOwnSlot];
      float p[kOwnPerLane][3];
#pragma unroll
      for (int j = 0; j < kOwnPerLane; ++j) {
        const int i = lane + 32 * j;
        const float4 o = (U.blk * kBlockPts + i < g.n_own) ? os[i] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (xform) {
          p[j][0] = (m[0] * o.x + m[1] * o.y + m[2] * o.z + m[9]) * sc;
          p[j][1] = (m[3] * o.x + m[4] * o.y + m[5] * o.z + m[10]) * sc;
          p[j][2] = (m[6] * o.x + m[7] * o.y + m[8] * o.z + m[11]) * sc;
        } else {
          p[j][0] = o.x * sc;
          p[j][1] = o.y * sc;
          p[j][2] = o.z * sc;
        }
      }
      pack_owned(p, q);
    }
    const PrepOut pb = ops.prep(sm, cur.stage, len, meta);
    const float4* __restrict__ bufA = pb.a;
    const float4* __restrict__ bufB = pb.b;
#pragma unroll 8  // independent element chains (as the single-pair sweeps)
    for (int c = warp; c < len; c += kWarps) {
      const float4 a = bufA[c];
      const float4 b = bufB[c];
#pragma unroll
      for (int k = 0; k < kPairs; ++k) elem(acc[k], q[k], a, b);
    }
    __syncthreads();
    cur = nx;
  }
  float tot[NACC];
  reduce_warps<NACC>(sm, acc, tot);
  if (split_complete<NACC>(sm, g, U.blk, U.sl, U.ph.geo_round, part, cnt, tot)) ops.fin(U.blk, tot, meta);
  return true;
}

// Every phase sweeps both clouds scaled by its exponent's factor sc (owned
// points when loaded, streamed ones in the prepare step), and the Softassign
// phases fold 2^c0 (wsc) into the streamed weights, so that the elements are
// EmicpElemScaled / SinkElemScaled / FinalElemScaled.

// E-step: the streamed X' times sc.
__device__ __forceinline__ PrepOut prep_scaled(SweepSmem& sm, int stage, int len, float sc) {
  for (int c = threadIdx.x; c < len; c += kThreads) {
    const float4 x = sm.raw[stage][c];
    sm.prep[c] = make_float4(x.x * sc, x.y * sc, x.z * sc, 0.f);
  }
  __syncthreads();
  return PrepOut{sm.prep, sm.prep};
}

// Streamed Y' posed by (R, t') = meta[0..11]: sc (R y' + t') and w wsc, with w
// from the stage's weights, or 1.
__device__ __forceinline__ PrepOut prep_posed(SweepSmem& sm, int stage, int len, const float* m, bool unit_weight,
                                              float sc, float wsc) {
  const float* w = reinterpret_cast<const float*>(&sm.raw2[stage][0]);
  for (int c = threadIdx.x; c < len; c += kThreads) {
    const float4 y = sm.raw[stage][c];
    sm.prep[c] = make_float4((m[0] * y.x + m[1] * y.y + m[2] * y.z + m[9]) * sc,
                             (m[3] * y.x + m[4] * y.y + m[5] * y.z + m[10]) * sc,
                             (m[6] * y.x + m[7] * y.y + m[8] * y.z + m[11]) * sc, (unit_weight ? 1.f : w[c]) * wsc);
  }
  __syncthreads();
  return PrepOut{sm.prep, sm.prep};
}

// Streamed X' for a column pass: (sc x', a_r wsc) with a from the completed row pass.
__device__ __forceinline__ PrepOut prep_weighted(SweepSmem& sm, int stage, int len, float sc, float wsc) {
  const float* w = reinterpret_cast<const float*>(&sm.raw2[stage][0]);
  for (int c = threadIdx.x; c < len; c += kThreads) {
    const float4 x = sm.raw[stage][c];
    sm.prep[c] = make_float4(x.x * sc, x.y * sc, x.z * sc, w[c] * wsc);
  }
  __syncthreads();
  return PrepOut{sm.prep, sm.prep};
}

// Streamed Y' for the final sweep: (sc (R y' + t'), b wsc) and
// (g (y' - Yhat), b (cs - 1) wsc) with g = b cs wsc, from the completed last
// column pass; Yhat = meta[28..30].
__device__ __forceinline__ PrepOut prep_final(SweepSmem& sm, int stage, int len, const float* m, float sc, float wsc) {
  const float* w = reinterpret_cast<const float*>(&sm.raw2[stage][0]);
  for (int c = threadIdx.x; c < len; c += kThreads) {
    const float4 y = sm.raw[stage][c];
    const float bn = w[c], csv = w[kChunk + c];
    const float g = bn * csv * wsc;
    sm.prep[c] = make_float4((m[0] * y.x + m[1] * y.y + m[2] * y.z + m[9]) * sc,
                             (m[3] * y.x + m[4] * y.y + m[5] * y.z + m[10]) * sc,
                             (m[6] * y.x + m[7] * y.y + m[8] * y.z + m[11]) * sc, bn * wsc);
    sm.prep2[c] = make_float4(g * (y.x - m[28]), g * (y.y - m[29]), g * (y.z - m[30]), bn * (csv - 1.f) * wsc);
  }
  __syncthreads();
  return PrepOut{sm.prep, sm.prep2};
}

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

// Per-phase operations of a sweep unit. meta: state floats [0..15] (R, t',
// sigma_p2 or T at [12]), centring header [16..31] (oX, oY, xmean, ymean).
// e = exp(-d^2 / (2 sigma_p2)) = 2^-|sc x - sc z|^2, sc = sqrt(log2(e) / (2 sigma_p2))
__device__ __forceinline__ float em_scale(float s2) { return sqrtf(kLog2e / (2.f * s2)); }

struct EmOps {  // EM-ICP E-step
  using Elem = EmicpElemScaled;
  const BPair* P;
  df* scratch;
  __device__ __forceinline__ Elem elem(const float*) const { return Elem{}; }
  __device__ __forceinline__ float scale(const float* m) const { return em_scale(m[12]); }
  __device__ __forceinline__ PrepOut prep(SweepSmem& sm, int stage, int len, const float* m) const {
    return prep_scaled(sm, stage, len, em_scale(m[12]));
  }
  __device__ __forceinline__ void fin(int blk, const float (&tot)[5], const float* m) const {
    const float inv_sc = 1.f / em_scale(m[12]);  // the e x sums came out sc times too large
    const float t5[5] = {tot[0], tot[1], tot[2] * inv_sc, tot[3] * inv_sc, tot[4] * inv_sc};
    const EmicpFin f{P->own0, P->M, expf(-P->d_02 / m[12]),  // src/emicp.cu:489
                     {m[24], m[25], m[26]}, nullptr, {m[16], m[17], m[18]}, scratch, P->rec};
    f(blk, t5);
  }
};

// K = exp((alpha - d^2)/T) / sqrt(T) = 2^c0 2^-|sc x - sc y|^2, sc = sqrt(log2(e) / T)
__device__ __forceinline__ float sa_scale(float T) { return sqrtf(kLog2e / T); }
__device__ __forceinline__ float sa_wscale(float alpha, float T) {
  const float kk = kLog2e / T;
  return exp2f(fmaf(alpha, kk, -0.5f * log2f(T)));
}

struct RowOps {  // Sinkhorn row pass k
  using Elem = SinkElemScaled;
  const BPair* P;
  bool first;
  __device__ __forceinline__ Elem elem(const float*) const { return Elem{}; }
  __device__ __forceinline__ float scale(const float* m) const { return sa_scale(m[12]); }
  __device__ __forceinline__ PrepOut prep(SweepSmem& sm, int stage, int len, const float* m) const {
    return prep_posed(sm, stage, len, m, first, sa_scale(m[12]), sa_wscale(P->alpha, m[12]));
  }
  __device__ __forceinline__ void fin(int blk, const float (&tot)[1], const float*) const {
    const BRowFin f{P->a, P->s, P->rs, P->N, first};
    f(blk, tot);
  }
};

struct ColOps {  // Sinkhorn column pass k
  using Elem = SinkElemScaled;
  const BPair* P;
  bool first, last;
  df* scratch;
  __device__ __forceinline__ Elem elem(const float*) const { return Elem{}; }
  __device__ __forceinline__ float scale(const float* m) const { return sa_scale(m[12]); }
  __device__ __forceinline__ PrepOut prep(SweepSmem& sm, int stage, int len, const float* m) const {
    return prep_weighted(sm, stage, len, sa_scale(m[12]), sa_wscale(P->alpha, m[12]));
  }
  __device__ __forceinline__ void fin(int blk, const float (&tot)[1], const float*) const {
    const BColFin f{P->b, P->u, P->cs, P->M, first, last, P->own1, scratch, P->rec + (size_t)P->g0.nblk * 32};
    f(blk, tot);
  }
};

struct FinOps {  // Softassign final sweep
  using Elem = FinalElemScaled;
  const BPair* P;
  df* scratch;
  __device__ __forceinline__ Elem elem(const float*) const { return Elem{}; }
  __device__ __forceinline__ float scale(const float* m) const { return sa_scale(m[12]); }
  __device__ __forceinline__ PrepOut prep(SweepSmem& sm, int stage, int len, const float* m) const {
    return prep_final(sm, stage, len, m, sa_scale(m[12]), sa_wscale(P->alpha, m[12]));
  }
  __device__ __forceinline__ void fin(int blk, const float (&tot)[5], const float*) const {
    const FinalFin f{P->own0, P->a, nullptr, P->N, scratch, P->rec};
    f(blk, tot);
  }
};

// ---------------------------------------------------------------- pose tasks
// Horn solve + pose store by thread 0; the carried eigenbasis lives in the
// pair's state block between solves.
__device__ __noinline__ void horn_update(const BPair& P, const float S[9], const float Xcp[3], const float Yd[3], int step,
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

__device__ __noinline__ void em_finalize(const BPair& P, const Ph& ph, df* s_red, df* s_tot) {
  __shared__ float s_emS[15];
  reduce_block_partials<kEmNV>(P.rec, P.g0.nblk, s_red, s_tot);
  em_moments_to_S_block(s_tot, s_emS);
  if (threadIdx.x == 0) {
    float Xc[3], Yc[3], S[9];
    for (int k = 0; k < 9; ++k) S[k] = s_emS[k];
    for (int k = 0; k < 3; ++k) {
      Xc[k] = s_emS[9 + k];
      Yc[k] = s_emS[12 + k];
    }
    horn_update(P, S, Xc, Yc, ph.step, ph.step + 1 == P.nsteps);
    __stcg(P.state + 12, __ldcg(P.state + 12) * P.sigma_factor);  // FP32, src/emicp.cu:668
  }
  __syncthreads();
}

__device__ __noinline__ void sa_finalize(const BPair& P, const Ph& ph, df* s_red, df* s_tot, float* s_S, float* s_v) {
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
  __shared__ float s_meta[32];
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
  // Units of a round: block b starts with unit b; further units are handed
  // out by the round's counter. Thread 0 requests one unit ahead, so the
  // atomic's latency is hidden behind the current unit (and the first request
  // of a round is issued before the previous round's barrier).
  __shared__ int s_next;
  __shared__ UnitRef s_cur;
  __shared__ Task s_tn;
  unsigned pending = 0;  // thread 0: next unit of this round
  if (tid == 0) pending = (unsigned)G + atomicAdd(&A.rctr[0], 1u);
  for (int r = 0; r < A.rounds && ok; ++r) {
    // Weights copied by TMA this round were written by other blocks in earlier
    // rounds (generic proxy, ordered by the grid barrier); the proxy fence
    // makes them visible to the async proxy of the copies thread 0 issues.
    if (tid == 0 && r > 0) asm volatile("fence.proxy.async.global;" ::: "memory");
    round_prefix(s_sched, A.npairs, r, s_pref);
    const int total = s_pref[A.npairs];
    int u = blockIdx.x;
    if (u < total) {
      Slot slot{0, 0u, false};
      {
        const Task t0 = first_task(resolve(A.pairs, s_sched, s_pref, A.npairs, r, u));
        if (t0.src) slot = ring_issue(rg, sm, t0);
      }
      for (;;) {
        // The unit and the next unit's first copy are block-uniform: thread 0
        // resolves them into shared memory (read where used, not held in
        // registers across the streaming loop).
        if (tid == 0) {
          const int nxt = (int)min(pending, 0x7fffffffu);
          pending = (unsigned)G + atomicAdd(&A.rctr[r], 1u);
          s_next = nxt;
          s_cur = resolve(A.pairs, s_sched, s_pref, A.npairs, r, u);
          s_tn = nxt < total ? first_task(resolve(A.pairs, s_sched, s_pref, A.npairs, r, nxt))
                             : Task{nullptr, 0, 0, nullptr, nullptr, nullptr, 0, nullptr, nullptr};
        }
        __syncthreads();
        const UnitRef& cur = s_cur;
        const int un = s_next;
        const Task& tn = s_tn;
        const BPair& P = A.pairs[cur.p];
        Slot ns{0, 0u, false};
        if (cur.ph.phase == kPhEmZ || cur.ph.phase == kPhSaZ) {
          if (tn.src) ns = ring_issue(rg, sm, tn);  // lands while the pose is solved
          if (cur.ph.phase == kPhEmZ) em_finalize(P, cur.ph, s_red, s_tot);
          else sa_finalize(P, cur.ph, s_red, s_tot, s_S, s_v);
        } else {
          df* scratch = reinterpret_cast<df*>(sm.prep);
          static_assert(offsetof(SweepSmem, full) - offsetof(SweepSmem, prep) >= 32 * (kBlockPts + 8) * sizeof(df),
                        "moment scratch does not fit");
          const BPair* PP = &A.pairs[cur.p];
          const int k = cur.ph.k;
          if (cur.ph.phase == kPhEmE)
            ok = run_sweep_unit<5>(sm, rg, cur, true, slot, tn, ns, P.part, P.cnt0, EmOps{PP, scratch}, s_meta,
                                   A.ctl, A.timeout_ns, 10);
          else if (cur.ph.phase == kPhSaRow)
            ok = run_sweep_unit<1>(sm, rg, cur, false, slot, tn, ns, P.part, P.cnt0, RowOps{PP, k == 0}, s_meta,
                                   A.ctl, A.timeout_ns, 30);
          else if (cur.ph.phase == kPhSaCol)
            ok = run_sweep_unit<1>(sm, rg, cur, true, slot, tn, ns, P.part, P.cnt1,
                                   ColOps{PP, k == 0, k == P.I1 - 1, scratch}, s_meta, A.ctl, A.timeout_ns, 40);
          else
            ok = run_sweep_unit<5>(sm, rg, cur, false, slot, tn, ns, P.part, P.cnt0, FinOps{PP, scratch}, s_meta,
                                   A.ctl, A.timeout_ns, 50);
        }
        if (!ok || un >= total) break;
        u = un;
        slot = ns;
      }
    }
    if (tid == 0 && r + 1 < A.rounds) pending = (unsigned)G + atomicAdd(&A.rctr[r + 1], 1u);
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

SweepGeom batch_geom(int n_own, int n_stream, int slice) {
  SweepGeom g{};
  g.n_own = n_own;
  g.n_stream = n_stream;
  g.nblk = (n_own + kBlockPts - 1) / kBlockPts;
  int S = (n_stream + slice - 1) / slice;
  if (S < 1) S = 1;
  g.slice_len = (((n_stream + S - 1) / S) + 3) & ~3;  // slices start at multiples of 4 points
  g.slices = (n_stream + g.slice_len - 1) / g.slice_len;
  g.units = g.nblk * g.slices;
  return g;
}

// Lays out the workspace: control block, all split counters (cleared per
// launch), the pair table, then each pair's buffers. With base == nullptr
// only sizes are computed.
// Slice length for a batch on a grid of G blocks: the largest sweep round
// (sum of N M over the pairs) in about kUnitsPerBlock * G units of 128 owned
// points, in whole TMA chunks.
int batch_slice(const BatchLaunchPair* in, int npairs, int G) {
  double work = 0.0;
  for (int i = 0; i < npairs; ++i) work += (double)in[i].N * (double)in[i].M;
  double chunks = work / (kUnitsPerBlock * (double)G * kBlockPts * kChunk);
  int c = (int)(chunks + 0.5);
  if (c < 1) c = 1;
  if (c > kMaxSliceChunks) c = kMaxSliceChunks;
  return c * kChunk;
}

// Lays out the workspace: control block, all split counters and the round
// counters (cleared per launch), the pair table, then each pair's buffers.
// The pair table is ordered by decreasing size, so the largest units of a
// round are handed out first. With base == nullptr only sizes are computed.
size_t carve_batch(void* base, const BatchLaunchPair* in, int npairs, int G, std::vector<BPair>* out, Ctl** ctl,
                   size_t* zero_bytes, BPair** dpairs, int* rounds, unsigned** rctr) {
  Carve c(base);
  *ctl = c.take<Ctl>(1);
  const int slice = batch_slice(in, npairs, G);
  std::vector<int> order((size_t)npairs);
  for (int i = 0; i < npairs; ++i) order[(size_t)i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (double)in[a].N * in[a].M > (double)in[b].N * in[b].M;
  });
  std::vector<BPair> v((size_t)npairs);
  size_t ncnt = 0;
  int rmax = 0;
  for (int i = 0; i < npairs; ++i) {
    const BatchLaunchPair& L = in[order[(size_t)i]];
    BPair& P = v[(size_t)i];
    P = BPair{};
    P.algo = L.algo;
    P.N = L.N;
    P.M = L.M;
    if (L.algo == 0) {
      P.g0 = batch_geom(L.M, L.N, slice);
      P.g1 = SweepGeom{0, 0, 0, 1, 0, 0};
      P.nsteps = L.nsteps;
      P.rounds = 2 * L.nsteps;
      P.init = L.sigma_p2;
      P.sigma_factor = L.sigma_factor;
      P.d_02 = L.d_02;
      P.I0 = 1;
      P.I1 = 1;
    } else {
      P.g0 = batch_geom(L.N, L.M, slice);
      P.g1 = batch_geom(L.M, L.N, slice);
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
    if (P.rounds > rmax) rmax = P.rounds;
  }
  unsigned* cnt = c.take<unsigned>(ncnt > 0 ? ncnt : 1);
  *rctr = c.take<unsigned>((size_t)rmax + 1);
  *zero_bytes = c.off;
  *dpairs = c.take<BPair>((size_t)npairs);
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
      // padded to 4 floats: weight copies are whole 16-byte groups
      const size_t Np = ((size_t)P.N + 3) & ~size_t(3), Mp = ((size_t)P.M + 3) & ~size_t(3);
      P.a = c.take<float>(Np);
      P.s = c.take<float>(Np);
      P.rs = c.take<float>(Np);
      P.b = c.take<float>(Mp);
      P.u = c.take<float>(Mp);
      P.cs = c.take<float>(Mp);
    }
    P.state = c.take<float>(kStateFloats);
  }
  if (out) out->swap(v);
  *rounds = rmax;
  return c.off;
}

size_t batch_smem(int npairs) {
  return sizeof(SweepSmem) + sizeof(Sched) * (size_t)npairs + sizeof(int) * ((size_t)npairs + 1);
}

}  // namespace

size_t batch_ws_need(const BatchLaunchPair* pairs, int npairs, int device) {
  Ctl* ctl = nullptr;
  size_t zb = 0;
  BPair* dp = nullptr;
  int rounds = 0;
  unsigned* rctr = nullptr;
  const int G = persistent_grid_limit(device, (const void*)batch_kernel, batch_smem(npairs));
  return carve_batch(nullptr, pairs, npairs, G, nullptr, &ctl, &zb, &dp, &rounds, &rctr);
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
  unsigned* rctr = nullptr;
  const size_t smem = batch_smem(npairs);
  const int limit = persistent_grid_limit(device, (const void*)batch_kernel, smem);
  const size_t need = carve_batch(ws, pairs, npairs, limit, &host, &ctl, &zero_bytes, &dpairs, &rounds, &rctr);
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
  if (grid_used) *grid_used = limit;
  if (rounds == 0) return 0;
  BatchArgs A;
  A.pairs = dpairs;
  A.npairs = npairs;
  A.rounds = rounds;
  A.rctr = rctr;
  A.ctl = ctl;
  A.d_status = d_status;
  A.timeout_ns = timeout_ns;
  void* args[] = {(void*)&A};
  e = cudaLaunchCooperativeKernel((const void*)batch_kernel, dim3(limit), dim3(kThreads), args, smem, st);
  return (int)e;
}

}  // namespace cesa
