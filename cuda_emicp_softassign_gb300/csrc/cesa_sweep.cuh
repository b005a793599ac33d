// Persistent "sweep" machinery shared by the EM-ICP and Softassign kernels.
//
// Both algorithms reduce a dense N x M affinity over one index: a row sum, a
// column sum, or a weighted row moment. The affinity is never stored. A sweep
// partitions the work into units of (128 owned points) x (a slice of streamed
// points):
//   * owned points live in registers, 4 per lane, 32 lanes -> 128 per unit;
//   * streamed points are brought into shared memory by 1-D TMA bulk copies
//     (cp.async.bulk, 2-stage ring, mbarrier completion) in chunks of 512.
//     The 8 warps split each chunk and every lane reads the same float4
//     (a broadcast);
//   * per-owned-point accumulators are reduced across the 8 warps through
//     shared memory in a fixed order.
// When a block of owned points is split over S > 1 slices, every unit stores
// its partial accumulators. The unit that finishes the block last (atomic
// counter per block, monotonic across sweeps) sums the S partials in slice
// order and runs the finalize step. Results are therefore deterministic
// whatever the scheduling.
//
// Units are assigned round-robin to the blocks of the persistent grid. The
// host picks S so that the unit count is close to a multiple of the grid size.
// Large clouds take the ranged decomposition instead (SweepGeom::ranged): each
// block a contiguous run of (owned block, chunk) tasks, the same work to one
// chunk, its deferred partials in per-(owned block, covering block) slots.
// A prepare step that copies its chunk into a buffer of its own can be
// double-buffered (prep_double_buffered): one block barrier per chunk.
#pragma once
#include <type_traits>

#include "cesa_common.cuh"

namespace cesa {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kOwnPerLane = 4;
constexpr int kBlockPts = 32 * kOwnPerLane;  // owned points per unit
constexpr int kChunk = 512;                  // streamed points per TMA chunk
constexpr int kStages = 2;
constexpr int kMaxAcc = 5;

// Geometry of one sweep type (host-computed).
struct SweepGeom {
  int n_own;      // owned points (rows of the reduction)
  int n_stream;   // streamed points
  int nblk;       // ceil(n_own / kBlockPts)
  int slices;     // S
  int slice_len;  // ceil(n_stream / S)
  int units;      // nblk * S
  // Ranged decomposition (deferred sweeps only; 0 = units of (owned block,
  // slice) dealt round-robin). The work is nblk * nch tasks of (owned block,
  // streamed chunk), in owned-block-major order; block b of the grid takes
  // the contiguous tasks [T b / G, T (b + 1) / G). Every block gets the same
  // work to one chunk, and a block meets an owned block only 2-3 times in a
  // sweep of a large cloud. Owned block o is covered by the consecutive grid
  // blocks b_lo(o) .. b_hi(o); the partials of the j-th of them are stored in
  // slot (o, j), j < kmax. Slots that no block writes (j > b_hi - b_lo) hold
  // zeros, set once per launch, so a consumer sums all kmax slots of a point
  // in slot order (the grid blocks' task order) with no division: adding +0
  // leaves a sum that starts at +0 bitwise unchanged.
  int ranged;
  int nch;        // ceil(n_stream / kChunk)
  int kmax;       // most grid blocks covering one owned block
  // SM pairs (ranged only; 0 = off). The G blocks are P = G / 2 pairs, two on
  // each SM, and pair d takes the tasks [T d / P, T (d + 1) / P), split at
  // pair_num / kPairDen of their count: virtual block 2 d the first part,
  // 2 d + 1 the rest. The partition, and so every slot's contents, is fixed;
  // which block of the pair computes which part is chosen at run time (the
  // block its SM favours takes the larger part: join_sm_pair, pair_swap).
  // Where a "block" b indexes tasks and slots below, it is the virtual index.
  int pair_num;
};

constexpr int kPairDen = 256;
constexpr int kPairCap = 1024;  // SM ids a pairing table covers

// The split point of a pair's tasks [lo, hi).
__host__ __device__ __forceinline__ long pair_split(long lo, long hi, int pair_num) {
  return lo + ((hi - lo) * pair_num + kPairDen / 2) / kPairDen;
}

// Task range [t0, t1) of block b in a ranged sweep over G blocks.
__host__ __device__ __forceinline__ void ranged_tasks(const SweepGeom& g, int b, int G, long& t0, long& t1) {
  const long T = (long)g.nblk * g.nch;
  if (g.pair_num) {
    const int P = G / 2, d = b >> 1;
    const long lo = T * d / P, hi = T * (d + 1) / P, sp = pair_split(lo, hi, g.pair_num);
    t0 = (b & 1) ? sp : lo;
    t1 = (b & 1) ? hi : sp;
    return;
  }
  t0 = T * b / G;
  t1 = T * (b + 1) / G;
}

// The grid block whose task range holds `task`: the largest b with
// floor(T b / G) <= task, i.e. floor(((task + 1) G - 1) / T).
__host__ __device__ __forceinline__ int ranged_block_of(const SweepGeom& g, long task, int G) {
  const long T = (long)g.nblk * g.nch;
  if (g.pair_num) {  // the pair, then the part
    const int P = G / 2;
    const int d = (int)(((task + 1) * (long)P - 1) / T);
    const long lo = T * d / P, hi = T * (d + 1) / P;
    return 2 * d + (task >= pair_split(lo, hi, g.pair_num) ? 1 : 0);
  }
  return (int)(((task + 1) * (long)G - 1) / T);
}

// One grid block's share of a ranged sweep: owned blocks [o_first, o_last]
// (o_last = -1: none), chunks [c_first, nch) of the first and [0, c_end) of the
// last, and j_first, its index among the blocks covering o_first (it is the
// first to cover every later owned block of its range). Computed once per
// launch (the 64-bit divisions stay out of the sweeps).
struct RangedShare {
  int o_first, o_last, c_first, c_end, j_first;
};

__device__ __forceinline__ RangedShare ranged_share(const SweepGeom& g, int b, int G) {
  RangedShare r{0, -1, 0, 0, 0};
  if (!g.ranged) return r;
  long t0 = 0, t1 = 0;
  ranged_tasks(g, b, G, t0, t1);
  if (t1 <= t0) return r;
  r.o_first = (int)(t0 / g.nch);
  r.o_last = (int)((t1 - 1) / g.nch);
  r.c_first = (int)(t0 - (long)r.o_first * g.nch);
  r.c_end = (int)(t1 - (long)r.o_last * g.nch);
  r.j_first = b - ranged_block_of(g, (long)r.o_first * g.nch, G);
  return r;
}

// SM pairs. With two blocks on an SM the warp scheduler favours the block it
// started first: the other mostly fills the first one's idle issue slots, and
// runs at full speed only once the first is done, so equal shares leave the SM
// half-used for the last part of every sweep. Thread 0 of each block joins its
// SM's pair: table [2 kPairCap + 1] (zero at launch) counts the blocks seen
// per SM id, holds each SM's dense pair index + 1 and, last, the pairs so far.
// Returns (pair index, role: 0 for the first block on its SM), or (-1, -1)
// when the SM id is out of the table, a third block arrives on one SM or the
// first one's index did not appear within timeout_ns. The first arrival is
// taken to be the favoured block; pair_swap corrects that from the times.
static __device__ __noinline__ int2 join_sm_pair(unsigned* tab, uint64_t timeout_ns) {
  unsigned sm_id;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(sm_id));
  if (sm_id >= (unsigned)kPairCap) return make_int2(-1, -1);
  const unsigned r = atomicAdd(&tab[sm_id], 1u);
  if (r == 0u) {
    const unsigned d = atomicAdd(&tab[2 * kPairCap], 1u);
    red_release_add(&tab[kPairCap + sm_id], d + 1u);  // the slot was 0
    return make_int2((int)d, 0);
  }
  if (r != 1u) return make_int2(-1, -1);
  uint64_t t0 = 0;
  unsigned spins = 0;
  for (;;) {
    const unsigned v = ld_acquire(&tab[kPairCap + sm_id]);
    if (v != 0u) return make_int2((int)v - 1, 1);
    if ((++spins & 31u) == 0) {
      const uint64_t now = global_ns();
      if (t0 == 0) {
        t0 = now;
      } else if (now - t0 > timeout_ns) {
        return make_int2(-1, -1);
      }
    }
  }
}

// Whether pair d's parts should change blocks: both parts hold work and the
// first part's sweep (time t[2 d], ns) took over 1.5 times the second's
// (t[2 d + 1]). Both blocks of the pair read the same two times after a grid
// barrier, so they agree.
__device__ __forceinline__ bool pair_swap(long lo, long split, long hi, const float* t, int d) {
  const float t0 = __ldcg(t + 2 * d), t1 = __ldcg(t + 2 * d + 1);
  return split > lo && hi > split && t0 > 1.5f * t1;
}

// Large sweeps take the ranged decomposition: at least 16 tasks per block, so
// that the one-chunk remainder is small.
__host__ __forceinline__ bool ranged_pays(int nblk, int n_stream, int G) {
  const long nch = (n_stream + kChunk - 1) / kChunk;
  return (long)nblk * nch >= 16L * G;
}

// The most grid blocks covering one owned block of a ranged geometry with
// g.nblk owned blocks of g.nch tasks each (host; g.nblk, g.nch >= 1).
__host__ __forceinline__ int ranged_kmax(const SweepGeom& g, int G) {
  int kmax = 1;
  for (int o = 0; o < g.nblk; ++o) {
    const int lo = ranged_block_of(g, (long)o * g.nch, G);
    const int hi = ranged_block_of(g, (long)(o + 1) * g.nch - 1, G);
    kmax = hi - lo + 1 > kmax ? hi - lo + 1 : kmax;
  }
  return kmax;
}

// Turns g into a ranged sweep over G blocks, tasks of kChunk streamed points
// (host; requires ranged_pays).
__host__ __forceinline__ void make_ranged(SweepGeom& g, int G) {
  g.ranged = 1;
  g.nch = (g.n_stream + kChunk - 1) / kChunk;
  g.kmax = ranged_kmax(g, G);
}

// Index of point i's first slot in a ranged partial array of one accumulator,
// [nblk][kmax][kBlockPts]; its slots follow kBlockPts apart.
__device__ __forceinline__ int ranged_slot0(int i, int kmax) {
  return ((i / kBlockPts) * kmax) * kBlockPts + (i % kBlockPts);
}

struct __align__(16) SweepSmem {
  float4 raw[kStages][kChunk];   // TMA destination, stream A
  float4 raw2[kStages][kChunk];  // TMA destination, stream B (optional)
  float4 prep[kChunk];           // prepared stream A (transformed / weighted)
  float4 prep2[kChunk];          // prepared stream B
  float red[kMaxAcc][kWarps][kBlockPts];
  uint64_t full[kStages];
  int flag;
};

// Per-block pipeline bookkeeping (identical in every thread of the block).
struct Pipe {
  unsigned uses[kStages];  // copies issued into each stage
  int tag[kStages];        // chunk id resident in each stage (static streams), -1 = none
  int cur;                 // stage of the task being consumed, -1 = none
  // first task of the next sweep, issued before the grid barrier that precedes it
  const float4* pre_src;
  int pre_stage, pre_first, pre_len;
  unsigned pre_par;
  bool pre_wait, pre_valid;
};

__device__ __forceinline__ void pipe_init(Pipe& p) {
  for (int s = 0; s < kStages; ++s) {
    p.uses[s] = 0;
    p.tag[s] = -1;
  }
  p.cur = -1;
  p.pre_valid = false;
}

// Owned points of the last unit a block processed in a sweep type, kept in
// shared memory (owned arrays never change during a launch).
struct OwnCache {
  float4 pts[kBlockPts];
  int blk;
};

// Streamed source for one sweep.
struct StreamSrc {
  const float4* a;  // required
  const float4* b;  // optional second array (same indexing), nullptr if unused
  bool is_static;   // contents never change during the launch (enables reuse)
};

// Chooses the stage for chunk `id`; issues the bulk copy unless a static
// chunk is already resident. Returns the stage; *need_wait tells the
// consumer whether to wait on the stage's mbarrier.
__device__ __forceinline__ int pipe_issue(Pipe& p, SweepSmem& sm, const StreamSrc& src, int id,
                                          int first, int len, bool& need_wait) {
  if (src.is_static) {
    for (int s = 0; s < kStages; ++s)
      if (p.tag[s] == id) {
        need_wait = false;
        return s;
      }
  }
  const int s = (p.cur < 0) ? 0 : (p.cur ^ 1);
  p.tag[s] = src.is_static ? id : -1;
  p.uses[s] += 1;
  need_wait = true;
  if (threadIdx.x == 0) {
    const unsigned bytes = (unsigned)len * 16u;
    mbar_arrive_expect_tx(&sm.full[s], src.b ? 2u * bytes : bytes);
    bulk_g2s(&sm.raw[s][0], src.a + first, bytes, &sm.full[s]);
    if (src.b) bulk_g2s(&sm.raw2[s][0], src.b + first, bytes, &sm.full[s]);
  }
  return s;
}

// Owned points of block `blk` from the cache, filling it from global memory on
// a miss (block-wide). Invalid points read as zero.
__device__ __forceinline__ void load_owned_cached(OwnCache& oc, const float4* own, int n_own, int blk,
                                                  float4 (&pt)[kOwnPerLane]) {
  if (oc.blk != blk) {  // uniform: every thread reads the same tag
    __syncthreads();
    if (threadIdx.x < kBlockPts) {
      const int i = blk * kBlockPts + (int)threadIdx.x;
      oc.pts[threadIdx.x] = i < n_own ? ld_cg(own + i) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    if (threadIdx.x == 0) oc.blk = blk;
  }
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < kOwnPerLane; ++j) pt[j] = oc.pts[lane + 32 * j];
}

// Owned-point loader: lane's 4 points of block `blk`. Invalid points get
// `fill` and valid=false.
__device__ __forceinline__ void load_owned(const float4* own, int n_own, int blk, float4 (&pt)[kOwnPerLane],
                                           bool (&valid)[kOwnPerLane]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < kOwnPerLane; ++j) {
    const int i = blk * kBlockPts + lane + 32 * j;
    valid[j] = i < n_own;
    pt[j] = valid[j] ? ld_cg(own + i) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Owned points of a lane in packed pairs: pair k holds the lane's points
// (2k, 2k + 1), i.e. owned indices lane + 64 k and lane + 64 k + 32.
constexpr int kPairs = kOwnPerLane / 2;

// Negated coordinates of the lane's owned points, packed by pair.
__device__ __forceinline__ void pack_owned(const float (&p)[kOwnPerLane][3], float2 (&q)[kPairs][3]) {
#pragma unroll
  for (int k = 0; k < kPairs; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) q[k][c] = make_float2(-p[2 * k][c], -p[2 * k + 1][c]);
}

// Writes the warp-level accumulators to shared memory and returns, in threads
// 0..kBlockPts-1, the sum over warps (fixed order) for owned point threadIdx.x.
// (Smem: any shared-memory block with red[kMaxAcc][kWarps][kBlockPts] and flag.)
template <int NACC, class Smem>
__device__ __forceinline__ void reduce_warps(Smem& sm, const float (&acc)[kOwnPerLane][NACC], float (&tot)[NACC]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < kOwnPerLane; ++j)
#pragma unroll
    for (int a = 0; a < NACC; ++a) sm.red[a][warp][lane + 32 * j] = acc[j][a];
  __syncthreads();
  if (threadIdx.x < kBlockPts) {
#pragma unroll
    for (int a = 0; a < NACC; ++a) {
      float s = sm.red[a][0][threadIdx.x];
#pragma unroll
      for (int w = 1; w < kWarps; ++w) s += sm.red[a][w][threadIdx.x];
      tot[a] = s;
    }
  }
  __syncthreads();
}

template <int NACC, class Smem>
__device__ __forceinline__ void reduce_warps(Smem& sm, const float2 (&acc)[kPairs][NACC], float (&tot)[NACC]) {
  float a[kOwnPerLane][NACC];
#pragma unroll
  for (int k = 0; k < kPairs; ++k)
#pragma unroll
    for (int v = 0; v < NACC; ++v) {
      a[2 * k][v] = acc[k][v].x;
      a[2 * k + 1][v] = acc[k][v].y;
    }
  reduce_warps<NACC>(sm, a, tot);
}

// Split-slice completion. Stores this unit's per-point totals; returns true in
// every thread of the block that must finalize block `blk`, with `tot` (threads
// < kBlockPts) replaced by the slice-ordered sum over all S partials.
// part layout: [(blk*S + sl)][NACC][kBlockPts]. cnt[blk] is monotonic; this is
// the `round`-th sweep of this geometry in the launch (0-based).
template <int NACC, class Smem>
__device__ __forceinline__ bool split_complete(Smem& sm, const SweepGeom& g, int blk, int sl,
                                               unsigned round, float* part, unsigned* cnt,
                                               float (&tot)[NACC]) {
  if (g.slices == 1) return true;
  float* mine = part + ((size_t)blk * g.slices + sl) * NACC * kBlockPts;
  if (threadIdx.x < kBlockPts) {
#pragma unroll
    for (int a = 0; a < NACC; ++a) __stcg(mine + a * kBlockPts + threadIdx.x, tot[a]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned old = atom_acq_rel_add(&cnt[blk], 1u);
    const unsigned target = (round + 1u) * (unsigned)g.slices;
    sm.flag = (old + 1u == target) ? 1 : 0;
  }
  __syncthreads();
  const bool last = sm.flag != 0;
  if (last) {
    // All threads take (accumulator, point) pairs; the S partials of a pair
    // are loaded 8 at a time (independent loads in flight) and summed in
    // slice order.
    const float* base = part + (size_t)blk * g.slices * NACC * kBlockPts;
    for (int p = threadIdx.x; p < NACC * kBlockPts; p += kThreads) {
      const float* src = base + p;
      float s = 0.f;
      int k = 0;
      for (; k + 16 <= g.slices; k += 16) {
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = __ldcg(src + (size_t)(k + j) * NACC * kBlockPts);
#pragma unroll
        for (int j = 0; j < 16; ++j) s += v[j];
      }
      if (k < g.slices) {
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j)
          v[j] = (k + j < g.slices) ? __ldcg(src + (size_t)(k + j) * NACC * kBlockPts) : 0.f;
#pragma unroll
        for (int j = 0; j < 16; ++j) s += v[j];  // zero padding does not change the sum
      }
      reinterpret_cast<float*>(sm.red)[p] = s;  // red is free after reduce_warps
    }
    __syncthreads();
    if (threadIdx.x < kBlockPts) {
#pragma unroll
      for (int a = 0; a < NACC; ++a) tot[a] = reinterpret_cast<float*>(sm.red)[a * kBlockPts + threadIdx.x];
    }
  }
  __syncthreads();
  return last;
}

// Accumulates NV per-thread df values (threads that have none pass zeros) into
// the block accumulator acc[NV] held in shared memory (thread 0 adds).
template <int NV>
__device__ __forceinline__ void block_accumulate(df (&v)[NV], df* red, df* acc) {
  static_assert(NV <= kThreads, "one thread per value");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const df o = df_shfl_down(v[k], off);
      df_add(v[k], o);
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) red[k * kWarps + warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < NV) {  // value k summed over the warps by thread k, fixed order
    df s = red[threadIdx.x * kWarps];
#pragma unroll
    for (int w = 1; w < kWarps; ++w) df_add(s, red[threadIdx.x * kWarps + w]);
    df_add(acc[threadIdx.x], s);
  }
  __syncthreads();
}

// Sum over the 128 owned points of NV per-point df values (thread i < 128
// holds point i; other threads pass zeros or nothing), written to dst[NV] in
// global memory. Goes through shared memory (`scratch`, >= NV*128 dfs) in
// a fixed order: 8 partial sums of 16 points per value, then 8 -> 1.
template <int NV>
__device__ __forceinline__ void owned_block_sum(const df (&v)[NV], df* scratch, df* dst) {
  static_assert(NV * 8 <= kThreads * 2, "two passes of the block at most");
  if (threadIdx.x < kBlockPts) {
#pragma unroll
    for (int k = 0; k < NV; ++k) scratch[k * kBlockPts + threadIdx.x] = v[k];
  }
  __syncthreads();
  df* part = scratch + NV * kBlockPts;  // [NV][8]
  for (int p = threadIdx.x; p < NV * 8; p += kThreads) {
    const int k = p >> 3, g = p & 7;
    const df* src = scratch + k * kBlockPts + g * 16;
    df s = src[0];
#pragma unroll
    for (int j = 1; j < 16; ++j) df_add(s, src[j]);
    part[p] = s;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    df s = part[threadIdx.x * 8];
#pragma unroll
    for (int g = 1; g < 8; ++g) df_add(s, part[threadIdx.x * 8 + g]);
    __stcg(reinterpret_cast<float2*>(dst + threadIdx.x), make_float2(s.hi, s.lo));
  }
  __syncthreads();
}

// Grid-wide sum of NV block partials (df), identical in every block: thread 0
// of the calling block receives the totals in tot[]. parts: [nblocks][NV].
__host__ __device__ constexpr int pow2_ceil(int v) { return v <= 1 ? 1 : 2 * pow2_ceil((v + 1) / 2); }

template <int NV>
__device__ __forceinline__ void reduce_block_partials(const df* parts, int nblocks, df* scratch,
                                                      df* tot) {
  constexpr int NVP = pow2_ceil(NV);  // lanes per group (values >= NV idle)
  constexpr int G = kThreads / NVP;   // threads per value
  static_assert(NVP <= 32, "at most 32 values");
  const int v = threadIdx.x % NVP, grp = threadIdx.x / NVP;
  const bool live = v < NV;
  // blocks grp, grp + G, ... in order; loads issued 8 at a time
  df a = df_make(0.f);
  int b = grp;
  for (; b + 7 * G < nblocks; b += 8 * G) {
    float2 x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      x[j] = live ? __ldcg(reinterpret_cast<const float2*>(parts + (size_t)(b + j * G) * NV + v))
                  : make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 8; ++j) df_add(a, df{x[j].x, x[j].y});
  }
  for (; b < nblocks; b += G) {
    const float2 x = live ? __ldcg(reinterpret_cast<const float2*>(parts + (size_t)b * NV + v))
                          : make_float2(0.f, 0.f);
    df_add(a, df{x.x, x.y});
  }
  // fixed tree over the groups: lanes of a warp with the same v, then warps
#pragma unroll
  for (int off = 16; off >= NVP; off >>= 1) {
    const df o = df_shfl_down(a, off);
    df_add(a, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane < NVP) scratch[warp * NVP + lane] = a;
  __syncthreads();
  if (threadIdx.x < NV) {
    df s = scratch[threadIdx.x];
#pragma unroll
    for (int w = 1; w < kWarps; ++w) df_add(s, scratch[w * NVP + threadIdx.x]);
    tot[threadIdx.x] = s;
  }
  __syncthreads();
}

// Streams as seen by the element function after the prepare step.
struct PrepOut {
  const float4* a;
  const float4* b;
};

// A prepare step that copies each chunk into its own double buffer (and does
// not read the stream stage after it returns, nor end with a barrier) sets
// kDoubleBuffered: its sweep then needs one block barrier per chunk, after
// the prepare step, and warps run one chunk apart (a warp may prepare chunk
// n + 1 while others still sweep chunk n from the other buffer).
template <class P, class = void>
struct prep_double_buffered : std::false_type {};
template <class P>
struct prep_double_buffered<P, std::void_t<decltype(P::kDoubleBuffered)>> : std::bool_constant<P::kDoubleBuffered> {};

// Prepare step that uses the streams as loaded.
struct NoPrep {
  __device__ __forceinline__ PrepOut operator()(SweepSmem& sm, int stage, int, int, int) const {
    return PrepOut{sm.raw[stage], sm.raw2[stage]};
  }
  __device__ __forceinline__ void unit_end(int, int) const {}
};

// Finalize step of a deferred sweep: the owned totals stay in the partial
// buffer and are combined by the consumer of the next sweep.
struct NoFin {
  template <int NACC>
  __device__ __forceinline__ void operator()(int, const float (&)[NACC]) const {}
};

// Issues, ahead of a sweep, the bulk copy of the first streamed chunk this
// block will need in it. Called block-wide after the previous sweep's last
// unit, before the grid barrier, so the copy lands while the barrier waits.
// Only for streams whose contents are final at that point (the coordinate
// arrays, which never change during a launch).
__device__ __forceinline__ void sweep_prefetch(Pipe& p, SweepSmem& sm, const SweepGeom& g,
                                               const StreamSrc& src) {
  const int u = blockIdx.x;
  if (p.pre_valid) return;
  int first = 0, len = 0;
  if (g.ranged) {  // the first task of this block's range
    long t0 = 0, t1 = 0;
    ranged_tasks(g, u, (int)gridDim.x, t0, t1);
    if (t1 <= t0) return;
    first = (int)(t0 % g.nch) * kChunk;
    len = min(kChunk, g.n_stream - first);
  } else {
    if (u >= g.units) return;
    const int sl = u % g.slices;
    const int sb = sl * g.slice_len;
    const int se = min(sb + g.slice_len, g.n_stream);
    first = sb;
    len = min(kChunk, se - sb);
  }
  p.cur = -1;
  bool w = false;
  const int st = pipe_issue(p, sm, src, first, first, len, w);
  p.pre_src = src.a;
  p.pre_stage = st;
  p.pre_par = (p.uses[st] - 1u) & 1u;
  p.pre_first = first;
  p.pre_len = len;
  p.pre_wait = w;
  p.pre_valid = true;
}

// Runs all units of one sweep assigned to this block (round-robin over the
// grid). For every unit: owned points -> registers (optionally transformed by
// R, tc), streamed chunks through the TMA ring, elem() per (owned, streamed)
// pair, cross-warp reduction, split completion, then fin(blk, tot) in the
// block that completes the owned block. Returns false if a wait gave up.
//
//   Elem: void operator()(float2 (&acc)[NACC], const float2 (&q)[3], float4 a, float4 b)
//         (two owned points, packed; q = their negated coordinates)
//   Prep: PrepOut operator()(SweepSmem&, int stage, int first, int len, int blk)  (block-wide)
//         void unit_end(int blk, int slice)                                       (block-wide)
//   Fin:  void operator()(int blk, const float (&tot)[NACC])                      (block-wide)
// kDeferred: the owned totals of slice sl are stored at part[sl * part_ld + point]
// and nothing is finalized here (no completion counter, no Fin); the sweep
// that streams these points next sums the S slices itself.
// kLayout: 1 for a ranged geometry (rs: this block's share of it, from
// ranged_share), 0 for units of (owned block, slice), -1 to read g.ranged at
// run time (a fixed layout keeps only its own bookkeeping live in registers).
template <int NACC, class Elem, class Prep, class Fin, bool kDeferred = false, int kLayout = -1>
__device__ __forceinline__ bool sweep_units(SweepSmem& sm, Pipe& pipe, const SweepGeom& g,
                                            const StreamSrc& src, const float4* own, bool xform_own,
                                            const float (&R)[9], const float (&tc)[3], unsigned round,
                                            float* part, unsigned* cnt, const Elem& elem,
                                            const Prep& prep, const Fin& fin, Ctl* ctl,
                                            uint64_t timeout_ns, int where, Timeline& tl,
                                            int part_ld = 0, OwnCache* oc = nullptr,
                                            const RangedShare* rs = nullptr) {
  const int tid = threadIdx.x, warp = tid >> 5;
  const int G = (int)gridDim.x;
  const bool ranged = kLayout < 0 ? g.ranged != 0 : kLayout == 1;
  constexpr bool kDB = prep_double_buffered<Prep>::value;
  pipe.cur = -1;
  // ranged: u is this block's segment index, and segment u covers chunks
  // [cb, ce) of owned block o_first + u: chunks [c_first, nch) of the first,
  // [0, c_end) of the last (o_last = -1 for an empty range). The share is read
  // from shared memory where it is used, not held in registers.
  auto task_range = [&](int uu, int ch, int& first, int& len) -> bool {
    if (ranged) {
      const int o = rs->o_first + uu;
      const int o_last = rs->o_last;
      if (o > o_last) return false;
      const int cb = uu == 0 ? rs->c_first : 0;
      const int ce = o == o_last ? rs->c_end : g.nch;
      const int c = cb + ch;
      if (c >= ce) return false;
      first = c * kChunk;
      len = min(kChunk, g.n_stream - first);
      return true;
    }
    if (uu >= g.units) return false;
    const int sl = uu % g.slices;
    const int sb = sl * g.slice_len;
    const int se = min(sb + g.slice_len, g.n_stream);
    first = sb + ch * kChunk;
    if (first >= se) return false;
    len = min(kChunk, se - first);
    return true;
  };
  const int ustep = ranged ? 1 : G;
  int u = ranged ? 0 : (int)blockIdx.x;
  int cur_first = 0, cur_len = 0, cur_ch = 0, cur_stage = 0;
  unsigned cur_par = 0;
  bool cur_wait = false;
  bool have = task_range(u, 0, cur_first, cur_len);
  const bool pre_hit = have && pipe.pre_valid && pipe.pre_src == src.a && pipe.pre_first == cur_first &&
                       pipe.pre_len == cur_len;
  if (pipe.pre_valid && !pre_hit && pipe.pre_wait) {  // unused prefetch: let it land
    if (!mbar_wait(&sm.full[pipe.pre_stage], pipe.pre_par, ctl, timeout_ns, where + 2)) {
      pipe.pre_valid = false;
      return false;
    }
  }
  if (pre_hit) {
    cur_stage = pipe.pre_stage;
    cur_par = pipe.pre_par;
    cur_wait = pipe.pre_wait;
  } else if (have) {
    cur_stage = pipe_issue(pipe, sm, src, cur_first, cur_first, cur_len, cur_wait);
    cur_par = (pipe.uses[cur_stage] - 1u) & 1u;
  }
  pipe.pre_valid = false;
  while (have) {
    const int blk = ranged ? rs->o_first + u : u / g.slices, sl = ranged ? u : u % g.slices;
    float4 ow[kOwnPerLane];
    if (oc) {
      load_owned_cached(*oc, own, g.n_own, blk, ow);
    } else {
      bool valid[kOwnPerLane];
      load_owned(own, g.n_own, blk, ow, valid);
    }
    float p[kOwnPerLane][3];
#pragma unroll
    for (int j = 0; j < kOwnPerLane; ++j) {
      if (xform_own) {
        p[j][0] = R[0] * ow[j].x + R[1] * ow[j].y + R[2] * ow[j].z + tc[0];
        p[j][1] = R[3] * ow[j].x + R[4] * ow[j].y + R[5] * ow[j].z + tc[1];
        p[j][2] = R[6] * ow[j].x + R[7] * ow[j].y + R[8] * ow[j].z + tc[2];
      } else {
        p[j][0] = ow[j].x;
        p[j][1] = ow[j].y;
        p[j][2] = ow[j].z;
      }
    }
    float2 q[kPairs][3];
    pack_owned(p, q);
    float2 acc[kPairs][NACC];
#pragma unroll
    for (int k = 0; k < kPairs; ++k)
#pragma unroll
      for (int a = 0; a < NACC; ++a) acc[k][a] = make_float2(0.f, 0.f);

    for (;;) {
      int n_first = 0, n_len = 0, n_u = u, n_ch = cur_ch + 1, n_stage = 0;
      unsigned n_par = 0;
      bool n_wait = false;
      bool have_n = task_range(n_u, n_ch, n_first, n_len);
      if (!have_n) {
        n_u = u + ustep;
        n_ch = 0;
        have_n = task_range(n_u, 0, n_first, n_len);
      }
      pipe.cur = cur_stage;
      if (have_n) {
        n_stage = pipe_issue(pipe, sm, src, n_first, n_first, n_len, n_wait);
        n_par = (pipe.uses[n_stage] - 1u) & 1u;
      }
      const bool bad = cur_wait && !mbar_wait(&sm.full[cur_stage], cur_par, ctl, timeout_ns, where);
      if (!kDB && __syncthreads_or(bad)) {  // block-uniform decision
        // leave only after the prefetched copy (if any) has landed
        if (have_n && n_wait) mbar_wait(&sm.full[n_stage], n_par, ctl, timeout_ns, where + 1);
        return false;
      }
      if (cur_ch == 0 && u == (int)blockIdx.x) tl.mark(2);
      // (double-buffered: a stage that timed out is read as it is; the
      // decision to leave is taken at the barrier after the prepare step)
      const PrepOut pb = prep(sm, cur_stage, cur_first, cur_len, blk);
      if (kDB && __syncthreads_or(bad)) {
        if (have_n && n_wait) mbar_wait(&sm.full[n_stage], n_par, ctl, timeout_ns, where + 1);
        return false;
      }
      const float4* __restrict__ bufA = pb.a;
      const float4* __restrict__ bufB = pb.b;
// 8 streamed points per iteration: independent element chains for the
      // scheduler (measured: C3 +7%, C5 +7%, the batch +8% over 2; 16 adds nothing)
#pragma unroll 8
      for (int c = warp; c < cur_len; c += kWarps) {
        const float4 a = bufA[c];
        const float4 b = bufB[c];
#pragma unroll
        for (int k = 0; k < kPairs; ++k) elem(acc[k], q[k], a, b);
      }
      if (!kDB) __syncthreads();  // the stage and the prepared chunk are consumed
      const bool unit_done = !(have_n && n_u == u);
      cur_first = n_first;
      cur_len = n_len;
      cur_ch = n_ch;
      cur_stage = n_stage;
      cur_par = n_par;
      cur_wait = n_wait;
      have = have_n;
      if (unit_done) break;
    }
    tl.mark(3);
    prep.unit_end(blk, sl);
    float tot[NACC];
    reduce_warps<NACC>(sm, acc, tot);
    if (kDeferred) {
      const int i = blk * kBlockPts + (int)threadIdx.x;
      if (threadIdx.x < kBlockPts && i < g.n_own) {
        if (ranged) {  // slot (owned block, j): this block is the j-th to cover it
          const int j = sl == 0 ? rs->j_first : 0;
          if (j < g.kmax) {
#pragma unroll
            for (int a = 0; a < NACC; ++a)
              __stcg(part + (((size_t)a * g.nblk + blk) * g.kmax + j) * kBlockPts + threadIdx.x, tot[a]);
          } else {
            set_status(ctl, kStatusInternal, where + 3);  // the plan's kmax is inconsistent
          }
        } else {
#pragma unroll
          for (int a = 0; a < NACC; ++a) __stcg(part + ((size_t)a * g.slices + sl) * part_ld + i, tot[a]);
        }
      }
    } else if (split_complete<NACC>(sm, g, blk, sl, round, part, cnt, tot)) {
      fin(blk, tot);
    }
    tl.mark(4);
    u += ustep;
    cur_ch = 0;
  }
  return true;
}

}  // namespace cesa
