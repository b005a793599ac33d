// Softassign, banded matrix-free form (sm_103a): the whole annealing schedule
// of softassign() (src/softassign.cu:486-822) in one persistent cooperative
// launch of thread-block clusters, for clouds of up to 2048 columns (Y points).
//
// The same arithmetic as the matrix-free kernel (M_rc = K_rc a_r b_c, K
// recomputed in every sweep, never stored), with another decomposition:
//  - The X rows are cut into bands of 64 and the Y columns into CS tiles of
//    W <= 256 (CS = 1, 2, 4 or 8). Band i is one cluster of CS CTAs; CTA j of
//    it holds the tile (band i, columns of tile j) for the whole launch: its
//    rows and columns stay in shared memory, there is no streaming. The
//    launch needs all nb = ceil(N / 64) clusters resident at once (on GB300,
//    36 clusters of 8 CTAs of this kernel: N <= 2304 at M > 1024).
//  - Row pass: each CTA sums K b over its tile's columns for the band's rows;
//    the cluster adds the CS partials through distributed shared memory (in
//    rank order) and every CTA of the band completes the pass for all of the
//    band's rows (rs, a, s) itself. A row pass therefore ends at a cluster
//    barrier, not at a grid barrier.
//  - Column pass: each CTA sums K a over the band's rows for its tile's
//    columns and stores the partial; after a barrier over the nb CTAs holding
//    tile j (a counter per tile, not the grid), each of them adds the nb band
//    partials of its columns (in band order) and completes the pass (cs, b, u)
//    itself.
//  - Final row sweep: w, mu and Vhat over the tile, added across the cluster;
//    the band's rows are finalised by the cluster's CTAs in 64 / CS row
//    shares and the tiles' columns in shares c = band (mod nb); their 28 row
//    and 4 column moments are added across the cluster by rank 0 into one
//    record per band.
//    One grid barrier, then every CTA reduces the nb records and solves the
//    pose.
// Per pose update: I1 tile-group barriers, 1 grid barrier and I1 + 2 cluster
// barriers, against 2 I1 + 1 grid barriers in the matrix-free kernel. Row-side state (a, s) is
// held, identical, by every CTA of a band and column-side state (b, u) by
// every CTA of a tile column, so no pass writes a scaling vector to global
// memory. Results agree with the matrix-free kernel to FP32 rounding (other
// summation orders), not bitwise.
//
// Cluster barriers have no time limit: every CTA runs the same sequence of
// them whatever happens. A grid or tile-group barrier that gives up (time
// limit, or a status already set by another CTA) only turns off the rest of
// this CTA's work.
#include <mutex>

#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_sa_pose.cuh"

namespace cesa {

struct BandArgs {
  const float4* rows;  // X' centred (N)
  const float4* cols;  // Y' centred (M)
  const CenterHdr* hdr;
  float* dRt;
  int N, M, Mp;
  int nb, CS, W;       // bands, CTAs per cluster (column tiles), tile width
  int JMAX, I0, I1;
  float alpha, T0, TFACTOR, moutlier;
  const float* s_in;   // optional initial slack [N] (else moutlier)
  const float* u_in;   // optional [M]
  float* s_out;        // optional final slack, row sums, column sums, w
  float* u_out;
  float* rs_out;
  float* cs_out;
  float* w_out;
  float* pc;           // column-pass partials [2][nb][Mp] (by pass parity)
  df* mom;             // [2][nb][32] moment records per band
  unsigned* gbar;      // [CS][32]: barrier counter of each column tile's nb CTAs (one 128-byte line each)
  Ctl* ctl;
  double* trace;
  int trace_cap;
  int* d_status;
  unsigned long long* tl;
  int tl_cap;
  uint64_t timeout_ns;
};

// Band height and tile width: the lanes own 2 rows (one packed pair) in row
// sweeps and 8 columns (four pairs) in column sweeps, so a CTA's tile holds up
// to 64 x 256 affinities, as many as one 128 x 128 unit of the matrix-free
// kernel, and 8-CTA clusters (the portable size) cover 2048 columns.
constexpr int kBandRows = 64;
constexpr int kTileCols = 256;
constexpr int kRowPairs = kBandRows / 64;
constexpr int kColPairs = kTileCols / 64;
constexpr int kMaxCluster = 8;
constexpr int kBandRed = kMaxAcc * kBandRows > kTileCols ? kMaxAcc * kBandRows : kTileCols;
// The tile's affinities K[c][r], computed by the first row pass of every
// inner iteration and read by its other 2 I1 sweeps (K depends on the pose and
// T only). Column stride 65: the row sweeps read 32 consecutive rows of a
// column, the column sweeps one row of 32 columns 65 apart, both without bank
// conflicts.
constexpr int kKld = kBandRows + 1;
static_assert(kWarps * kBandRed * sizeof(float) >= (32 * 32 + 32 * kWarps) * 8, "moment scratch");

struct __align__(16) BandSmem {
  float4 xr[kBandRows];   // the band's rows x' (fixed)
  float4 xs[kBandRows];   // column-sweep stream: (x', a_r)
  float4 yc[kTileCols];   // the tile's columns y' (fixed)
  float4 ys[kTileCols];   // row-sweep stream: (R y' + t', b_c)
  float4 ys2[kTileCols];  // final-sweep second stream: (g_c (y' - Yhat), delta_c)
  float a[kBandRows], s[kBandRows], rs[kBandRows];  // band rows
  float b[kTileCols], u[kTileCols], cs[kTileCols];  // tile columns
  float xpart[2][kMaxAcc][kBandRows];               // this CTA's row partials, read by the cluster
  df mrec[32];                                      // this CTA's moments, read by rank 0
  float red[kWarps * kBandRed];                     // cross-warp reduction scratch (also 32 x 40 dfs)
  float K[kTileCols * kKld];                        // the tile's affinities, column-major
};

// Row sweeps over the cached K: acc (rows lane, lane + 32) += K[c][r] w_c over
// the streamed columns c < len (w_c: the .w of sw[c], and for NACC = 5 also
// the second stream h[c]). With `store`, K is computed (e = 2^(cK + nk d^2),
// as in SinkElem) and written to the cache instead of read.
template <int NACC, bool kStore>
__device__ __forceinline__ void band_row_sweep(float* K, const float2 (&q)[3], float nk, float cK, const float4* sw,
                                               const float4* h, int len, float2 (&acc)[NACC]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll 8  // independent element chains (C2 76.1 -> 77.3 reg/s over 2)
  for (int c = warp; c < len; c += kWarps) {
    const float4 y = sw[c];
    float2 e;
    if (kStore) {
      e = ex2_pair(__ffma2_rn(dist2_pair(q, y), dup2(nk), dup2(cK)));
      K[c * kKld + lane] = e.x;
      K[c * kKld + lane + 32] = e.y;
    } else {
      e = make_float2(K[c * kKld + lane], K[c * kKld + lane + 32]);
    }
    acc[0] = __ffma2_rn(e, dup2(y.w), acc[0]);
    if (NACC == 5) {
      const float4 g = h[c];
      acc[1] = __ffma2_rn(e, dup2(g.w), acc[1]);
      acc[2] = __ffma2_rn(e, dup2(g.x), acc[2]);
      acc[3] = __ffma2_rn(e, dup2(g.y), acc[3]);
      acc[4] = __ffma2_rn(e, dup2(g.z), acc[4]);
    }
  }
}

// Column sweep over the cached K: acc (columns lane + 64 k, lane + 64 k + 32)
// += K[c][r] a_r over the streamed rows r < len (a_r: the .w of sx[r]).
__device__ __forceinline__ void band_col_sweep(const float* K, const float4* sx, int len,
                                               float2 (&acc)[kColPairs][1]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll 8
  for (int r = warp; r < len; r += kWarps) {
    const float a = sx[r].w;
#pragma unroll
    for (int k = 0; k < kColPairs; ++k) {
      const float2 e = make_float2(K[(lane + 64 * k) * kKld + r], K[(lane + 64 * k + 32) * kKld + r]);
      acc[k][0] = __ffma2_rn(e, dup2(a), acc[k][0]);
    }
  }
}

// Negated coordinates of the lane's owned points, packed: pair k holds points
// lane + 64 k and lane + 64 k + 32.
template <int P>
__device__ __forceinline__ void own_pairs(const float4* pts, float2 (&q)[P][3]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < P; ++k) {
    const float4 u = pts[lane + 64 * k];
    const float4 v = pts[lane + 64 * k + 32];
    q[k][0] = make_float2(-u.x, -v.x);
    q[k][1] = make_float2(-u.y, -v.y);
    q[k][2] = make_float2(-u.z, -v.z);
  }
}

// Sum over the 8 warps (fixed order) of the per-point accumulators; thread i
// < 64 P receives owned point i's totals. Synchronises the block.
template <int NACC, int P>
__device__ __forceinline__ void band_reduce(float* red, const float2 (&acc)[P][NACC], float (&tot)[NACC]) {
  constexpr int n = 64 * P;
  static_assert(NACC * n <= kBandRed, "reduction scratch");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < P; ++k)
#pragma unroll
    for (int a = 0; a < NACC; ++a) {
      red[(warp * NACC + a) * n + lane + 64 * k] = acc[k][a].x;
      red[(warp * NACC + a) * n + lane + 64 * k + 32] = acc[k][a].y;
    }
  __syncthreads();
  if (threadIdx.x < n) {
#pragma unroll
    for (int a = 0; a < NACC; ++a) {
      float s = red[a * n + threadIdx.x];
#pragma unroll
      for (int w = 1; w < kWarps; ++w) s += red[(w * NACC + a) * n + threadIdx.x];
      tot[a] = s;
    }
  }
  __syncthreads();
}

// Completion of column pass kk for the tile's columns (normalizeMbySinkhorn_col
// + Saxpy, src/softassign.cu:579-597): cs = b_old (column sum of K a) + u_old,
// b = b_old / cs, u = u_old / cs, b_old = 1 for the first pass of an inner
// iteration. The column sums are the nb band partials, added in band order.
// For the final sweep it also prepares the second stream.
__device__ __forceinline__ void band_complete_columns(const BandArgs& A, BandSmem& sm, const float* pc_pass,
                                                      int kk, int c0, int Wt, bool final_sweep, const float* yh) {
  const int tid = threadIdx.x;
  if (tid < Wt) {
    const float* P = pc_pass + c0 + tid;
    // the first 32 band partials all in flight before the first add (adding
    // the zeros of absent bands leaves the sum unchanged), then the rest
    float v[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = j < A.nb ? __ldcg(P + (size_t)j * A.Mp) : 0.f;
    float sum = 0.f;
#pragma unroll
    for (int j = 0; j < 32; ++j) sum += v[j];
    for (int i = 32; i < A.nb; ++i) sum += __ldcg(P + (size_t)i * A.Mp);
    const float bo = kk >= 1 ? sm.b[tid] : 1.f, uo = sm.u[tid];
    const float csv = fmaf(bo, sum, uo);
    const float bn = bo / csv;
    sm.b[tid] = bn;
    sm.u[tid] = uo / csv;
    sm.cs[tid] = csv;
    sm.ys[tid].w = bn;
    if (final_sweep) {
      const float g = bn * csv;
      const float4 y = sm.yc[tid];
      sm.ys2[tid] = make_float4(g * (y.x - yh[0]), g * (y.y - yh[1]), g * (y.z - yh[2]), bn * (csv - 1.f));
    }
  }
  __syncthreads();
}

// Sum over the CTA of the final moments, into dst[32] (shared), in a fixed
// order. v[] is non-zero only in threads 0..active-1 (the CTA's share of the
// band's rows and of the tiles' columns). Up to 32 active threads (every
// cluster of 2 or more CTAs with nb >= 8), through shared memory; else only the
// first active / 32 warps reduce by shuffles, level-major in groups of values.
// Synchronises the block.
__device__ __forceinline__ void band_moment_sum(df (&v)[32], int active, df* red, df* scratch, df* dst) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (active <= 32) {
    // through shared memory: value k of entry i at scratch[k * 32 + i]; thread
    // (k, g) = (tid % 32, tid / 32) adds entries g, g + 8, ... in order, then
    // thread k adds the 8 group sums in order
    df* part = scratch + 32 * 32;
    if ((int)threadIdx.x < active)
#pragma unroll
      for (int k = 0; k < 32; ++k) scratch[k * 32 + threadIdx.x] = v[k];
    __syncthreads();
    df sg = df_make(0.f);
    for (int i = warp; i < active; i += kWarps) df_add(sg, scratch[lane * 32 + i]);
    part[lane * kWarps + warp] = sg;
    __syncthreads();
    if (threadIdx.x < 32) {
      df s = part[threadIdx.x * kWarps];
#pragma unroll
      for (int w = 1; w < kWarps; ++w) df_add(s, part[threadIdx.x * kWarps + w]);
      dst[threadIdx.x] = s;
    }
    __syncthreads();
    return;
  }
  const int nw = (active + 31) >> 5;
  int top = 1;  // the smallest power of two >= min(active, 32)
  while (top < active && top < 32) top <<= 1;
  if (warp < nw) {
#pragma unroll
    for (int g = 0; g < 32; g += 8)
      for (int off = top >> 1; off > 0; off >>= 1) {
#pragma unroll
        for (int k = g; k < g + 8; ++k) {
          const df o = df_shfl_down(v[k], off);
          df_add(v[k], o);
        }
      }
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < 32; ++k) red[k * kWarps + warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int k = threadIdx.x;
    df s = df_make(0.f);
    for (int w = 0; w < nw; ++w) df_add(s, red[k * kWarps + w]);
    dst[k] = s;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kThreads, 2) softassign_band_kernel(const BandArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BandSmem& sm = *reinterpret_cast<BandSmem*>(smem_raw);
  __shared__ float s_pose[12];
  __shared__ float s_hdr[12];
  __shared__ df s_red[kThreads];
  __shared__ df s_tot[kSaNV];
  __shared__ SaPoseScratch ps;
  __shared__ HornState<float> horn;

  const int tid = threadIdx.x;
  const int CS = A.CS;
  // The kernel reads its peers' shared memory at ranks 0..CS-1: a launch whose
  // clusters do not hold CS CTAs (the same answer in every CTA of a cluster)
  // records an error and leaves before any cluster barrier or remote access.
  if (cluster_nctarank() != (unsigned)CS || cluster_id_x() >= (unsigned)A.nb) {
    if (tid == 0) set_status(A.ctl, kStatusUnsupported, 70);
    if (tid == 0 && blockIdx.x == 0 && A.d_status) *A.d_status = kStatusUnsupported;
    return;
  }
  const unsigned rank = cluster_ctarank();
  const int band = (int)cluster_id_x();
  const int r0 = band * kBandRows, c0 = (int)rank * A.W;
  const int Hb = min(kBandRows, A.N - r0);
  const int Wt = max(0, min(A.W, A.M - c0));
  const bool col_rec = band == 0;
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);

  static_assert(kTileCols == kThreads && kBandRows <= kThreads, "one thread per column");
  if (tid < kBandRows) {
    sm.xr[tid] = tid < Hb ? ld_cg(A.rows + r0 + tid) : zero4;
    sm.xs[tid] = zero4;
    sm.s[tid] = tid < Hb ? (A.s_in ? A.s_in[r0 + tid] : A.moutlier) : 0.f;
    sm.a[tid] = 1.f;
    sm.rs[tid] = 0.f;
  }
  sm.yc[tid] = tid < Wt ? ld_cg(A.cols + c0 + tid) : zero4;
  sm.ys2[tid] = zero4;
  sm.u[tid] = tid < Wt ? (A.u_in ? A.u_in[c0 + tid] : A.moutlier) : 0.f;
  sm.b[tid] = 1.f;
  sm.cs[tid] = 0.f;
  if (tid == 0) {
    for (int k = 0; k < 3; ++k) {
      s_hdr[k] = A.hdr->oX[k];
      s_hdr[3 + k] = A.hdr->oY[k];
      s_hdr[6 + k] = A.hdr->ymean[k];
    }
    float R[9], t[3], tc[3];
    for (int k = 0; k < 9; ++k) R[k] = A.dRt[k];
    for (int k = 0; k < 3; ++k) t[k] = A.dRt[9 + k];
    pose_to_centred(R, t, &s_hdr[0], &s_hdr[3], tc);
    for (int k = 0; k < 9; ++k) s_pose[k] = R[k];
    for (int k = 0; k < 3; ++k) s_pose[9 + k] = tc[k];
    horn.reset();
  }
  __syncthreads();
  float2 qx[kRowPairs][3];  // the band's rows, owned by the lanes in row sweeps
  own_pairs(sm.xr, qx);

  unsigned epoch = 0, gepoch = 0, cpass = 0;
  int xpar = 0, step = 0;
  bool ok = true;
  float T = A.T0;
  Timeline tl{A.tl, A.tl_cap, 0};
  const size_t pc_stride = (size_t)A.nb * A.Mp;

  for (int Titer = 0; Titer < A.JMAX; ++Titer) {
    // K = exp((alpha - d^2)/T) / sqrt(T) = 2^(cK + nk d^2)
    const float kk2 = kLog2e / T;
    const float nk = -kk2;
    const float cK = fmaf(A.alpha, kk2, -0.5f * log2f(T));
    for (int iter0 = 0; iter0 < A.I0; ++iter0, ++step) {
      tl.mark(1);
      float R[9], tc[3];
#pragma unroll
      for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
      {
        const float4 y = sm.yc[tid];
        sm.ys[tid] = tid < Wt ? make_float4(R[0] * y.x + R[1] * y.y + R[2] * y.z + tc[0],
                                            R[3] * y.x + R[4] * y.y + R[5] * y.z + tc[1],
                                            R[6] * y.x + R[7] * y.y + R[8] * y.z + tc[2], 1.f)
                              : zero4;
      }
      __syncthreads();
      for (int k = 0; k < A.I1; ++k) {
        if (k >= 1) {
          band_complete_columns(A, sm, A.pc + (size_t)((cpass - 1u) & 1u) * pc_stride, k - 1, c0, Wt, false,
                                nullptr);
          tl.mark(14);
        }
        // row pass k: sum over the tile of K b, added across the cluster
        float2 acc[kRowPairs][1];
#pragma unroll
        for (int q = 0; q < kRowPairs; ++q) acc[q][0] = make_float2(0.f, 0.f);
        if (ok) {
          if (k == 0)  // K for this inner iteration, into the cache
            band_row_sweep<1, true>(sm.K, qx[0], nk, cK, sm.ys, nullptr, Wt, acc[0]);
          else
            band_row_sweep<1, false>(sm.K, qx[0], nk, cK, sm.ys, nullptr, Wt, acc[0]);
        }
        float tot[1];
        band_reduce<1>(sm.red, acc, tot);
        if (tid < kBandRows) sm.xpart[xpar][0][tid] = tot[0];
        tl.mark(15);
        cluster_sync_all();
        tl.mark(8);
        // completion (normalizeMbySinkhorn_row + Saxpy, src/softassign.cu:538-561):
        // rs = a_old (row sum of K b) + s_old, a = a_old / rs, s = s_old / rs
        if (tid < Hb) {
          // all CS remote loads in flight before the first add (rank order kept)
          float pv[kMaxCluster];
#pragma unroll
          for (int j = 0; j < kMaxCluster; ++j) pv[j] = j < CS ? ld_dsmem(&sm.xpart[xpar][0][tid], (unsigned)j) : 0.f;
          float sum = pv[0];
#pragma unroll
          for (int j = 1; j < kMaxCluster; ++j)
            if (j < CS) sum += pv[j];
          const float ao = k >= 1 ? sm.a[tid] : 1.f, so = sm.s[tid];
          const float rsv = fmaf(ao, sum, so);
          const float an = ao / rsv;
          sm.a[tid] = an;
          sm.s[tid] = so / rsv;
          sm.rs[tid] = rsv;
          const float4 x = sm.xr[tid];
          sm.xs[tid] = make_float4(x.x, x.y, x.z, an);
        }
        xpar ^= 1;
        __syncthreads();
        tl.mark(3);
        // column pass k: sum over the band of K a, one partial per band
        float2 acc2[kColPairs][1];
#pragma unroll
        for (int q = 0; q < kColPairs; ++q) acc2[q][0] = make_float2(0.f, 0.f);
        if (ok) band_col_sweep(sm.K, sm.xs, Hb, acc2);
        band_reduce<1>(sm.red, acc2, tot);
        if (tid < Wt) __stcg(A.pc + (size_t)(cpass & 1u) * pc_stride + (size_t)band * A.Mp + c0 + tid, tot[0]);
        ++cpass;
        tl.mark(4);
        // the completion of tile `rank`'s columns reads only the partials of
        // the nb CTAs of that tile: a barrier over that group, not the grid
        if (ok) ok = counter_sync(A.gbar + (size_t)rank * 32, A.ctl, gepoch, (unsigned)A.nb, A.timeout_ns, 72);
        tl.mark(5);
      }
      // final row sweep: completes the last column pass, accumulates w, mu, Vhat
      band_complete_columns(A, sm, A.pc + (size_t)((cpass - 1u) & 1u) * pc_stride, A.I1 - 1, c0, Wt, true,
                            &s_hdr[6]);
      tl.mark(2);
      float2 acc5[kRowPairs][5];
#pragma unroll
      for (int q = 0; q < kRowPairs; ++q)
#pragma unroll
        for (int m = 0; m < 5; ++m) acc5[q][m] = make_float2(0.f, 0.f);
      if (ok) band_row_sweep<5, false>(sm.K, qx[0], nk, cK, sm.ys, sm.ys2, Wt, acc5[0]);
      float tot5[5];
      band_reduce<5>(sm.red, acc5, tot5);
      if (tid < kBandRows) {
#pragma unroll
        for (int m = 0; m < 5; ++m) sm.xpart[xpar][m][tid] = tot5[m];
      }
      cluster_sync_all();
      tl.mark(8);
      // this CTA's share of the band's rows: w = a K b, mu = a K delta,
      // Vhat = a K g (y' - Yhat), and their 28 moments
      df v[32];
#pragma unroll
      for (int m = 0; m < 32; ++m) v[m] = df_make(0.f);
      {
        const int share = (kBandRows + CS - 1) / CS;
        const int rb = (int)rank * share;
        const int re = min(rb + share, Hb);
        if (tid < re - rb) {
          const int r = rb + tid;
          float pv[kMaxCluster][5];
#pragma unroll
          for (int j = 0; j < kMaxCluster; ++j)
#pragma unroll
            for (int m = 0; m < 5; ++m) pv[j][m] = j < CS ? ld_dsmem(&sm.xpart[xpar][m][r], (unsigned)j) : 0.f;
          float t5[5];
#pragma unroll
          for (int m = 0; m < 5; ++m) {
            t5[m] = pv[0][m];
#pragma unroll
            for (int j = 1; j < kMaxCluster; ++j)
              if (j < CS) t5[m] += pv[j][m];
          }
          const float ar = sm.a[r];
          const float w = ar * t5[0], mu = ar * t5[1];
          const float V[3] = {ar * t5[2], ar * t5[3], ar * t5[4]};
          const float4 x = sm.xr[r];
          const float xp[3] = {x.x, x.y, x.z};
          if (A.w_out) A.w_out[r0 + r] = w;
          sa_row_moments(v, w, mu, V, xp);
        }
      }
      // the column moments sum cs, sum cs y' of the tile's columns c = band
      // (mod nb), so that every band takes a share of them
      const int ncols = Wt > band ? (Wt - band + A.nb - 1) / A.nb : 0;
      if (tid < ncols) {
        const int c = band + tid * A.nb;
        const float csv = sm.cs[c];
        const float4 y = sm.yc[c];
        df_add(v[28], csv);
        df_add_prod(v[29], csv, y.x);
        df_add_prod(v[30], csv, y.y);
        df_add_prod(v[31], csv, y.z);
      }
      xpar ^= 1;
      tl.mark(11);
      {
        const int share = (kBandRows + CS - 1) / CS;
        const int nrows = max(0, min(share, Hb - (int)rank * share));
        band_moment_sum(v, max(nrows, ncols), s_red, reinterpret_cast<df*>(sm.red), sm.mrec);
      }
      tl.mark(12);
      cluster_sync_all();
      tl.mark(10);
      df* rec = A.mom + (size_t)(step & 1) * A.nb * 32;
      if (rank == 0 && tid < 32) {
        df pv[kMaxCluster];
#pragma unroll
        for (int j = 0; j < kMaxCluster; ++j) pv[j] = j < CS ? ld_dsmem(&sm.mrec[tid], (unsigned)j) : df_make(0.f);
        df m = pv[0];
#pragma unroll
        for (int j = 1; j < kMaxCluster; ++j)
          if (j < CS) df_add(m, pv[j]);
        __stcg(reinterpret_cast<float2*>(rec + (size_t)band * 32 + tid), make_float2(m.hi, m.lo));
      }
      tl.mark(4);
      if (ok) ok = grid_sync(A.ctl, epoch, gridDim.x, A.timeout_ns, 74);
      tl.mark(5);
      if (ok) {
        reduce_block_partials<32>(rec, A.nb, s_red, s_tot);
        tl.mark(6);
        double* trace_rec = (A.trace && step < A.trace_cap) ? A.trace + (size_t)step * 32 : nullptr;
        sa_pose_update(s_tot, s_hdr, ps, horn, s_pose, blockIdx.x == 0, nullptr, trace_rec, step, T, A.ctl, &tl,
                       true);
      }
      tl.mark(7);
    }
    T = T * A.TFACTOR;  // FP32, src/softassign.cu:820
  }

  if (rank == 0 && tid < Hb) {
    if (A.s_out) A.s_out[r0 + tid] = sm.s[tid];
    if (A.rs_out) A.rs_out[r0 + tid] = sm.rs[tid];
  }
  if (col_rec && tid < Wt) {
    if (A.u_out) A.u_out[c0 + tid] = sm.u[tid];
    if (A.cs_out) A.cs_out[c0 + tid] = sm.cs[tid];
  }
  if (blockIdx.x == 0 && tid == 0) {
    const int st = ld_status(A.ctl);
    if (st == kStatusOk) {
      float R[9], tc[3], t[3];
      for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
      for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
      pose_from_centred(R, tc, &s_hdr[0], &s_hdr[3], t);
      for (int k = 0; k < 9; ++k) A.dRt[k] = R[k];
      for (int k = 0; k < 3; ++k) A.dRt[9 + k] = t[k];
    }
    if (A.d_status) *A.d_status = st;
    if (A.tl) A.ctl->pad[0] = (unsigned)tl.n;
  }
  cluster_sync_all();  // no CTA leaves while a peer may still read its shared memory
}

// ------------------------------------------------------------------ host side
namespace {

struct BandPlan {
  bool ok = false;
  int CS = 0, W = 0, nb = 0, grid = 0;
  size_t smem = 0;
};

// Thread-block clusters of CS CTAs of this kernel that fit on the device at
// once (queried once per device and cluster size).
int band_max_clusters(int device, int CS) {
  static std::mutex mu;
  static int cached[64][4];
  static bool init = false;
  std::lock_guard<std::mutex> lock(mu);
  if (!init) {
    for (auto& d : cached)
      for (int& v : d) v = -1;
    init = true;
  }
  int lg = 0;
  while ((1 << lg) < CS) ++lg;
  if (device < 0 || device >= 64 || lg > 3) return 0;
  if (cached[device][lg] >= 0) return cached[device][lg];
  const size_t smem = sizeof(BandSmem);
  cudaFuncSetAttribute((const void*)softassign_band_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CS);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CS;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (const void*)softassign_band_kernel, &cfg) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  cached[device][lg] = n;
  return n;
}

BandPlan plan_band(int N, int M, int device) {
  BandPlan P;
  if (N < 1 || M < 1) return P;
  int CS = 1;
  while (CS < kMaxCluster && (M + CS - 1) / CS > kTileCols) CS *= 2;
  const int W = (M + CS - 1) / CS;
  if (W > kTileCols) return P;
  const int nb = (N + kBandRows - 1) / kBandRows;
  if (nb > band_max_clusters(device, CS)) return P;
  P.ok = true;
  P.CS = CS;
  P.W = W;
  P.nb = nb;
  P.grid = nb * CS;
  P.smem = sizeof(BandSmem);
  return P;
}

struct BandCarved {
  Ctl* ctl;
  CenterHdr* hdr;
  float4* rows;
  float4* cols;
  float* pc;
  df* mom;
  unsigned* gbar;
  int Mp;
};

BandCarved carve_band(void* base, const BandPlan& P, int N, int M, size_t* total) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* p = base ? static_cast<char*>(base) + off : nullptr;
    off += (bytes + 255) & ~size_t(255);
    return p;
  };
  BandCarved w;
  w.Mp = (M + 3) & ~3;
  w.ctl = static_cast<Ctl*>(take(sizeof(Ctl)));
  w.hdr = static_cast<CenterHdr*>(take(sizeof(CenterHdr)));
  w.rows = static_cast<float4*>(take(sizeof(float4) * (size_t)N));
  w.cols = static_cast<float4*>(take(sizeof(float4) * (size_t)M));
  w.pc = static_cast<float*>(take(sizeof(float) * 2 * (size_t)P.nb * w.Mp));
  w.mom = static_cast<df*>(take(sizeof(df) * 2 * (size_t)P.nb * 32));
  w.gbar = static_cast<unsigned*>(take(sizeof(unsigned) * 32 * (size_t)P.CS));
  if (total) *total = off;
  return w;
}

}  // namespace

bool softassign_band_fits(int N, int M, int device) { return plan_band(N, M, device).ok; }

bool softassign_band_preferred(int N, int M, int device) {
  const BandPlan P = plan_band(N, M, device);
  if (!P.ok) return false;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  // enough CTAs to occupy the GPU, and few band partials per column
  return P.grid * 2 >= sms && P.nb <= 48;
}

size_t softassign_band_ws_need(int N, int M, int device) {
  const BandPlan P = plan_band(N, M, device);
  if (!P.ok) return 0;
  size_t total = 0;
  carve_band(nullptr, P, N, M, &total);
  return total;
}

int enqueue_softassign_band(const SoftassignLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  const BandPlan P = plan_band(L.N, L.M, device);
  if (!P.ok) return (int)cudaErrorInvalidConfiguration;
  size_t total = 0;
  BandCarved w = carve_band(ws, P, L.N, L.M, &total);
  if (total > ws_bytes) return (int)cudaErrorInvalidValue;
  if (grid_used) *grid_used = P.grid;
  e = cudaMemsetAsync(w.ctl, 0, sizeof(Ctl), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.gbar, 0, sizeof(unsigned) * 32 * (size_t)P.CS, st);
  if (e != cudaSuccess) return (int)e;
  prep_center_kernel<<<1, 1024, 0, st>>>(L.dX, L.N, L.dY, L.M, w.hdr);
  const int pb = 256, pg_x = (L.N + pb - 1) / pb, pg_y = (L.M + pb - 1) / pb;
  prep_pack_kernel<<<pg_x < 1024 ? pg_x : 1024, pb, 0, st>>>(L.dX, L.N, w.hdr, 0, 0.f, w.rows);
  prep_pack_kernel<<<pg_y < 1024 ? pg_y : 1024, pb, 0, st>>>(L.dY, L.M, w.hdr, 1, 0.f, w.cols);
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (L.JMAX <= 0 || L.I0 <= 0) return 0;
  BandArgs A;
  A.rows = w.rows;
  A.cols = w.cols;
  A.hdr = w.hdr;
  A.dRt = L.dRt;
  A.N = L.N;
  A.M = L.M;
  A.Mp = w.Mp;
  A.nb = P.nb;
  A.CS = P.CS;
  A.W = P.W;
  A.JMAX = L.JMAX;
  A.I0 = L.I0;
  A.I1 = L.I1;
  A.alpha = L.alpha;
  A.T0 = L.T_0;
  A.TFACTOR = L.TFACTOR;
  A.moutlier = L.moutlier;
  A.s_in = L.s_io;
  A.u_in = L.u_io;
  A.s_out = L.s_io;
  A.u_out = L.u_io;
  A.rs_out = L.rs_out;
  A.cs_out = L.cs_out;
  A.w_out = L.w_out;
  A.pc = w.pc;
  A.mom = w.mom;
  A.gbar = w.gbar;
  A.ctl = w.ctl;
  A.trace = L.trace;
  A.trace_cap = L.trace_cap;
  A.d_status = L.d_status;
  A.tl = L.timeline;
  A.tl_cap = L.timeline_cap;
  A.timeout_ns = L.timeout_ns;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(P.grid);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = P.smem;
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = P.CS;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeCooperative;
  at[1].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 2;
  return (int)cudaLaunchKernelEx(&cfg, softassign_band_kernel, A);
}

}  // namespace cesa
