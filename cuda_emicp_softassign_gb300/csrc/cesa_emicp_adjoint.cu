// Adjoint of the annealed EM-ICP registration for sm_103a: gradients of a
// loss of the final pose with respect to the clouds X, Y and the initial pose.
//
// The forward kernel records, per sigma step, its input pose, the 16 moments,
// the Horn eigenbasis and, per Y row, (C_r, lambda_r, u_r) (O(M) per step; no
// affinity is stored). One persistent launch walks the steps backwards:
//   1. every block: the O(1) adjoint of t' = Xc - R Yc, of R(q), of the top
//      eigenvector of Horn's N (sum over the other eigenvectors of
//      (v_j . gq) / (l_0 - l_j) v_j q^T), of N(S) and of the moment algebra,
//      giving dL/d(L, U, P, Q) for L = sum lambda, U = sum u, P = sum lambda y,
//      Q = sum u y^T;
//   2. one sweep that recomputes the affinities e_rc = exp(-|x_c - z_r|^2 / 2 s2)
//      (z_r = R y_r + t) over (column block, row slice) units. A lane owns 6
//      X columns; Y rows stream through shared memory as records of packed
//      row pairs (-z, the scaled row-sum adjoints, gB). Per element,
//      ge = gA_r + gB_r . x_c + 2 e gC_r (the adjoints of the row sums A = sum e,
//      B = sum e x, C = sum e^2 + outlier) and w = e ge / s2:
//        dL/dx_c += e gB_r - w (x_c - z_r)   (per column, in registers)
//        dL/dz_r += w (x_c - z_r)            (per row: summed over the lane's
//                                             columns, then over the lanes by a
//                                             ring of shuffles (each lane adds
//                                             its columns to the sum it receives
//                                             and passes it on), then over the
//                                             warps; one partial per column
//                                             block and row);
//   3. after a grid barrier every block completes a contiguous share of the
//      rows (all blocks at once, no serial tail): it sums the row partials in
//      column-block order, adds dL/dy_r = R^T dL/dz_r + lambda_r gP + gQ^T u_r
//      and writes its record of sum dL/dz_r y_r^T (row-major, as R),
//      sum dL/dz_r and, for rows on the C_r <= 1e-6 branch (lambda = 1,
//      u = mean X), sum gu_r;
//   4. after a second grid barrier every block reduces the records (the
//      upstream gradient of the previous step's pose) and adds, for its share
//      of the columns, the row-slice partials of dL/dx_c in a fixed order.
// Per element: 6 (distance) + 4 (ge, with 1/s2 folded into the row
// coefficients) + 3 (t = gB - ge (x - z) / s2) + 3 (dx += e t) + 3 (dz += e t)
// FP32 ops + 1 MUFU, against 12 + 1 in the forward, on packed pairs of rows
// (FFMA2/FADD2/FMUL2). The row sums carry e gB, which sums to gB A_r =
// gu_r lambda_r (A_r = sum_c e, lambda_r = A_r C_r^-1/2 from the tape) and is
// subtracted once per row at its completion.
#include <cstdlib>

#include "cesa.h"
#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {
namespace {

constexpr int kAdjCols = 6;                       // owned X columns per lane
constexpr int kAdjColBlk = kThreads * kAdjCols;   // owned columns per unit
constexpr int kAdjRows = kThreads;                // streamed Y rows per chunk (one record per thread)
constexpr int kAdjRP = kAdjRows / 2;              // row pairs per chunk
constexpr int kAdjGroups = kAdjRP / 32;           // groups of 32 row pairs (one per lane) per chunk
constexpr int kAdjRecStride = 14;                 // float2 per row-pair record (11 used; 112 bytes, so
                                                  // 8 lanes reading 8 consecutive records hit 32 banks)
constexpr float kFar = 1e15f;                     // padding row coordinate: its affinities are exactly 0
constexpr int kAdjPairNum = 192;                  // SM pairs, slices: the first 192/256 of a pair's units go
                                                  // to the block its SM favours
#ifndef CESA_ADJ_RANGED_PAIR
#define CESA_ADJ_RANGED_PAIR 193
#endif
constexpr int kAdjRangedPairNum = CESA_ADJ_RANGED_PAIR;  // SM pairs, ranged: the favoured block's share of tasks, /256
// Padding column coordinate, already scaled: its squared distance to any row
// (|z'| far below 2^26) is above 2^50, so its affinity is exactly 0, and its
// term ge (x - z) + gB stays finite (for row coefficients below 2^70), so that
// e times it is 0 and not 0 * inf.
constexpr float kPadScaled = 67108864.f;          // 2^26

// Units: nb column blocks x S row slices of len rows (even), slice-major.
// Ranged (large clouds): tasks of (column block, chunk of kAdjRows rows) in
// column-block-major order, block b taking the contiguous tasks
// [T b / G, T (b + 1) / G), as in the forward's ranged sweeps; the dL/dx
// partials of the j-th grid block covering column block cb go to slot
// (cb, j), j < kmax (slots no block writes stay zero from the launch).
struct AdjGeom {
  int nb, S, len, units;
  int ranged, nch, kmax;
  int pair_num;  // ranged: SM pairs (SweepGeom::pair_num), 0 = off
};

// The adjoint's ranged tasks in the sweep geometry that ranged_share reads.
__host__ __device__ inline SweepGeom adj_tasks(const AdjGeom& g) {
  SweepGeom t{};
  t.nblk = g.nb;
  t.nch = g.nch;
  t.ranged = g.ranged;
  t.pair_num = g.pair_num;
  return t;
}

struct EmAdjArgs {
  const float4* rows;  // Y' centred (M)
  const float4* cols;  // X' centred (N)
  int M, N;
  AdjGeom geo;
  int nsteps;
  const float* tape;      // [nsteps][kEmTape]
  const float* row_tape;  // [nsteps][M][5]
  const float* g_out;     // dL/d(R, t) of the final pose (device, caller frame)
  const CenterHdr* hdr;   // centring offsets (t' = t + R oY - oX)
  float4* gX;             // [N] accumulated (centred = caller frame)
  float4* gY;             // [M]
  float* g_in;            // [12] dL/d(R, t) of the initial pose, caller frame
  float4* part_z;         // [nb][M]: dL/dz per column block
  df* rec;                // [2][grid][16]: per-block records of the row completion
  float4* part_x;         // [2][S][N]: dL/dx per row slice; ranged: [2][nb][kmax][kAdjColBlk]
  Ctl* ctl;
  unsigned* pair_tab;  // [2 kPairCap + 1] (cleared): blocks seen per SM, pair index + 1 per SM, pairs so far
  float* pair_t;       // [grid]: sweep time of each (pair, part), ns
  int pairs;           // 1: units dealt to SM pairs (two blocks per SM, slice layout)
  int* d_status;
  uint64_t timeout_ns;
};

// ---------------------------------------------------------------- O(1) adjoint
// From the step's tape record and dL/d(R', t') of its output pose: the
// coefficients gL, gU[3], gP[3], gQ[9] (Q index i + 3 j = sum u_i y_j).
__device__ void em_step_adjoint(const float* rec, const float (&gRo)[9], const float (&gto)[3], float (&coef)[16]) {
  df m[kEmNV];
  for (int k = 0; k < kEmNV; ++k) m[k] = df{rec[16 + 2 * k], rec[17 + 2 * k]};
  float Xc[3], Yc[3], S[9];
  em_moments_to_S(m, Xc, Yc, S);
  const float L = df_val(m[0]);
  float q[4], V[4][4];
  for (int k = 0; k < 4; ++k) q[k] = rec[64 + k];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) V[i][j] = rec[48 + 4 * i + j];
  float gS[9], gXc[3], gYc[3];
  horn_pose_adjoint(S, Xc, Yc, q, V, gRo, gto, gS, gXc, gYc);
  // S[i + 3j] = Q[i + 3j] - L Xc_i Yc_j, Xc = U / L, Yc = P / L
  float gL = 0.f;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      const float g = gS[i + 3 * j];
      coef[7 + i + 3 * j] = g;  // gQ
      gL -= g * Xc[i] * Yc[j];
      gXc[i] -= L * g * Yc[j];
      gYc[j] -= L * g * Xc[i];
    }
  for (int i = 0; i < 3; ++i) {
    coef[1 + i] = gXc[i] / L;  // gU
    coef[4 + i] = gYc[i] / L;  // gP
    gL -= (gXc[i] * Xc[i] + gYc[i] * Yc[i]) / L;
  }
  coef[0] = gL;
}

// Per row: z (posed), and the row-sum adjoints gA, gB[3], gC (zero for
// rows on the C <= 1e-6 branch and for rows past M).
struct RowCoef {
  float z[3];
  float gA, gB[3], gC2;  // gC2 = 2 gC
};

__device__ __forceinline__ RowCoef row_coef(const float4 y, bool valid, const float* rt, const float* R,
                                            const float* t, const float* coef) {
  RowCoef c;
  c.z[0] = R[0] * y.x + R[1] * y.y + R[2] * y.z + t[0];
  c.z[1] = R[3] * y.x + R[4] * y.y + R[5] * y.z + t[1];
  c.z[2] = R[6] * y.x + R[7] * y.y + R[8] * y.z + t[2];
  c.gA = 0.f;
  c.gB[0] = c.gB[1] = c.gB[2] = 0.f;
  c.gC2 = 0.f;
  if (!valid) return c;
  const float C = rt[0];
  if (!(C > 10e-7f)) return c;  // src/emicp.cu:155 branch: no dependence on the affinities
  const float lam = rt[1];
  const float u[3] = {rt[2], rt[3], rt[4]};
  const float yy[3] = {y.x, y.y, y.z};
  float glam = coef[0], gu[3];
  for (int i = 0; i < 3; ++i) {
    glam += coef[4 + i] * yy[i];
    gu[i] = coef[1 + i] + coef[7 + i] * yy[0] + coef[10 + i] * yy[1] + coef[13 + i] * yy[2];
  }
  const float inv = rsqrtf(C);
  c.gA = glam * inv;
  for (int i = 0; i < 3; ++i) c.gB[i] = gu[i] * inv;
  c.gC2 = -(glam * lam + gu[0] * u[0] + gu[1] * u[1] + gu[2] * u[2]) / C;  // 2 gC
  return c;
}

struct AdjSmem {
  float2 rec[2][kAdjRP][kAdjRecStride];       // row-pair records, two chunks
  float wsum[2][3][kWarps][kAdjRows];         // per-warp row totals, two chunks
  df red[16 * kWarps];
};

// The record of one streamed row (one thread per row), in coordinates scaled
// by sc = sqrt(log2(e) / (2 s2)), so that e = 2^-|x' - z'|^2 needs no scale
// per element: -z', -gA/s2, -gB/(s2 sc), -2gC/s2 and gB sc, interleaved with
// the other row of its pair. (-gB/s2 multiplies the unscaled x = x'/sc; gB sc
// and the scaled differences make the sweep's dL/dx and dL/dz sc times the
// true ones, which the unit divides out once.)
__device__ __forceinline__ void build_row_record(AdjSmem& sm, int buf, int i, bool valid, float4 y, const float (&rt)[5],
                                                 const float* R, const float* t, const float* coef, float inv_s2,
                                                 float sc, float inv_sc) {
  float v[11];
  if (valid) {
    const RowCoef c = row_coef(y, true, rt, R, t, coef);
    v[0] = -c.z[0] * sc;
    v[1] = -c.z[1] * sc;
    v[2] = -c.z[2] * sc;
    v[3] = -c.gA * inv_s2;
    v[4] = -c.gB[0] * inv_s2 * inv_sc;
    v[5] = -c.gB[1] * inv_s2 * inv_sc;
    v[6] = -c.gB[2] * inv_s2 * inv_sc;
    v[7] = -c.gC2 * inv_s2;
    v[8] = c.gB[0] * sc;
    v[9] = c.gB[1] * sc;
    v[10] = c.gB[2] * sc;
  } else {  // far away, no coefficients: every term it feeds is 0
    v[0] = v[1] = v[2] = kFar;
#pragma unroll
    for (int k = 3; k < 11; ++k) v[k] = 0.f;
  }
  float* dst = reinterpret_cast<float*>(&sm.rec[buf][i >> 1][0]) + (i & 1);
#pragma unroll
  for (int k = 0; k < 11; ++k) dst[2 * k] = v[k];
}

// SM pairs (join_sm_pair): in the slice layout, where every unit owns its
// partial slots, the units of each SM's pair of blocks are split 12 : 4, the
// larger part to the block the SM favours, so that both finish together. The
// split decides which block computes a unit, never what the unit computes, so
// the results do not depend on it.
struct PairUnits {
  int lo, split, hi;  // part 0: [lo, split), part 1: [split, hi)
};

__host__ __device__ inline PairUnits pair_units(int units, int npairs, int d) {
  PairUnits r;
  r.lo = (int)((long long)units * d / npairs);
  r.hi = (int)((long long)units * (d + 1) / npairs);
  r.split = (int)pair_split(r.lo, r.hi, kAdjPairNum);
  return r;
}

// dL/dz of row r (of a chunk ending before row `end`) from one column block:
// the warps' row totals in warp order, unscaled, stored to the block's slot
__device__ __forceinline__ void complete_chunk_rows(const AdjSmem& sm, int buf, int r, int end, int cb, float inv_sc,
                                                    const EmAdjArgs& A) {
  if (r >= end) return;
  const int i = threadIdx.x;
  float gz[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float v = sm.wsum[buf][a][0][i];
#pragma unroll
    for (int w = 1; w < kWarps; ++w) v += sm.wsum[buf][a][w][i];
    gz[a] = -v * inv_sc;
  }
  __stcg(A.part_z + (size_t)cb * A.M + r, make_float4(gz[0], gz[1], gz[2], 0.f));
}

__global__ void __launch_bounds__(kThreads, 2) emicp_adjoint_kernel(const EmAdjArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  AdjSmem& sm = *reinterpret_cast<AdjSmem*>(smem_raw);
  __shared__ float s_g[12];     // dL/d(R, t') of the current step's output pose
  __shared__ float s_coef[16];  // moment adjoints of the current step
  __shared__ float s_pose[13];  // the step's input pose and sigma_p2
  __shared__ df s_red[kThreads];
  __shared__ df s_tot[16];
  __shared__ RangedShare rsh;  // this block's share of the ranged tasks
  __shared__ int s_pair[3];    // SM pairs: pair index, role, parts swapped
  __shared__ uint64_t s_tsweep;  // SM pairs: start of this step's sweep

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned G = gridDim.x;
  const AdjGeom& g = A.geo;
  if (tid == 0) {
    s_pair[0] = -1;
    int vb = (int)blockIdx.x;  // ranged: the virtual block whose share this block sweeps
    if (A.pairs || g.pair_num) {
      const int2 pr = join_sm_pair(A.pair_tab, A.timeout_ns);
      if (pr.x < 0 || pr.x >= (int)G / 2) set_status(A.ctl, kStatusInternal, 105);
      s_pair[0] = pr.x >= 0 && pr.x < (int)G / 2 ? pr.x : -1;
      s_pair[1] = pr.y;
      s_pair[2] = 0;
      vb = 2 * pr.x + pr.y;
    }
    rsh = g.pair_num && s_pair[0] < 0 ? RangedShare{0, -1, 0, 0, 0} : ranged_share(adj_tasks(g), vb, (int)G);
    // caller frame -> centred frame: t = t' + oX - R oY, so dL/dt' = dL/dt and
    // dL/dR' = dL/dR - dL/dt oY^T
    for (int i = 0; i < 3; ++i) {
      s_g[9 + i] = A.g_out[9 + i];
      for (int j = 0; j < 3; ++j) s_g[3 * i + j] = A.g_out[3 * i + j] - A.g_out[9 + i] * A.hdr->oY[j];
    }
  }
  __syncthreads();
  unsigned epoch = 0;
  bool ok = true;
  for (int k = A.nsteps - 1; k >= 0 && ok; --k) {
    const int par = k & 1;
    const float* rec = A.tape + (size_t)k * kEmTape;
    if (tid == 0) {
      float gRo[9], gto[3], coef[16];
      for (int i = 0; i < 9; ++i) gRo[i] = s_g[i];
      for (int i = 0; i < 3; ++i) gto[i] = s_g[9 + i];
      em_step_adjoint(rec, gRo, gto, coef);
      for (int i = 0; i < 16; ++i) s_coef[i] = coef[i];
      for (int i = 0; i < 13; ++i) s_pose[i] = rec[i];
    }
    __syncthreads();
    // the step's pose and coefficients stay in shared memory (read per row record)
    const float* R = s_pose;
    const float* t = s_pose + 9;
    const float* coef = s_coef;
    const float s2 = s_pose[12];
    const float inv_s2 = 1.f / s2;
    const float sc = sqrtf(kLog2e / (2.f * s2)), inv_sc = 1.f / sc;  // coordinate scale
    const float* rtape = A.row_tape + (size_t)k * A.M * 5;
    df* recs = A.rec + (size_t)par * G * 16;
    const size_t px_len = g.ranged ? (size_t)g.nb * g.kmax * kAdjColBlk : (size_t)g.S * A.N;
    float4* px = A.part_x + (size_t)par * px_len;

    int u_begin = (int)blockIdx.x, u_end = g.units, u_step = (int)G;
    if (g.ranged) {
      u_begin = 0;
      u_end = rsh.o_last - rsh.o_first + 1;
      u_step = 1;
    } else if (A.pairs) {  // this block's part of its pair's units (none after a failed join)
      u_begin = u_end = 0;
      u_step = 1;
      if (s_pair[0] >= 0) {
        const PairUnits pu = pair_units(g.units, (int)G / 2, s_pair[0]);
        const bool first = (s_pair[1] ^ s_pair[2]) == 0;
        u_begin = first ? pu.lo : pu.split;
        u_end = first ? pu.split : pu.hi;
      }
    }
    if (tid == 0 && s_pair[0] >= 0) s_tsweep = global_ns();
    for (int u = u_begin; u < u_end; u += u_step) {
      // unit: column block cb, rows [rb, re); its dL/dx partials go to px_dst
      int cb, rb, re;
      float4* px_dst;
      if (g.ranged) {  // segment u of this block's task run
        cb = rsh.o_first + u;
        const int c0 = u == 0 ? rsh.c_first : 0;
        const int c1 = cb == rsh.o_last ? rsh.c_end : g.nch;
        rb = c0 * kAdjRows;
        re = min(c1 * kAdjRows, A.M);
        const int j = u == 0 ? rsh.j_first : 0;
        // the slot must exist: an inconsistent plan records an error and
        // stores nothing (px_dst = nullptr) rather than writing past the array
        px_dst = j < g.kmax && cb < g.nb ? px + ((size_t)cb * g.kmax + j) * kAdjColBlk : nullptr;
        if (!px_dst && tid == 0) set_status(A.ctl, kStatusInternal, 104);
      } else {
        const int sl = u / g.nb;
        cb = u - sl * g.nb;
        rb = sl * g.len;
        re = min(rb + g.len, A.M);
        px_dst = px + (size_t)sl * A.N + (size_t)cb * kAdjColBlk;
      }
      // owned columns, duplicated into both halves of a packed pair
      float2 xd[kAdjCols][3], gx[kAdjCols][3];
#pragma unroll
      for (int j = 0; j < kAdjCols; ++j) {
        const int c = cb * kAdjColBlk + j * kThreads + tid;
        const float4 x = c < A.N ? ld_cg(A.cols + c) : make_float4(0.f, 0.f, 0.f, 0.f);
        xd[j][0] = dup2(c < A.N ? x.x * sc : kPadScaled);
        xd[j][1] = dup2(c < A.N ? x.y * sc : kPadScaled);
        xd[j][2] = dup2(c < A.N ? x.z * sc : kPadScaled);
#pragma unroll
        for (int a = 0; a < 3; ++a) gx[j][a] = make_float2(0.f, 0.f);
      }
      // the first chunk's row, loaded by its thread
      float4 yn = make_float4(0.f, 0.f, 0.f, 0.f);
      float rtn[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
      if (rb + tid < re) {
        yn = ld_cg(A.rows + rb + tid);
#pragma unroll
        for (int q = 0; q < 5; ++q) rtn[q] = __ldcg(rtape + (size_t)(rb + tid) * 5 + q);
      }
      // One barrier per chunk, records and row totals double-buffered: the
      // build of chunk n writes rec[n & 1], last read by the sweep of chunk
      // n - 2, which every warp finished before the barrier of chunk n - 1;
      // the sweep of chunk n writes wsum[n & 1], last read by the completion
      // of chunk n - 2, which every thread did before that same barrier; the
      // completion of chunk n - 1 reads wsum[(n - 1) & 1] after the barrier of
      // chunk n, by which time every warp has finished that sweep.
      __syncthreads();  // the previous unit's shared-memory use is over
      int buf = 0;
      for (int r0 = rb; r0 < re; r0 += kAdjRows, buf ^= 1) {
        build_row_record(sm, buf, tid, r0 + tid < re, yn, rtn, R, t, coef, inv_s2, sc, inv_sc);
        __syncthreads();
        if (r0 > rb) complete_chunk_rows(sm, buf ^ 1, r0 - kAdjRows + tid, r0, cb, inv_sc, A);
        // the next chunk's row, in flight during this chunk's sweep
        const int rn = r0 + kAdjRows + tid;
        if (rn < re) {
          yn = ld_cg(A.rows + rn);
#pragma unroll
          for (int q = 0; q < 5; ++q) rtn[q] = __ldcg(rtape + (size_t)rn * 5 + q);
        }
        // The warp's 32 lanes pass each row pair's dL/dz sum round a ring: at
        // step s lane l takes pair (l - s) mod 32 of every group of 32 pairs,
        // adds its columns' terms to the sum it received from lane l - 1 and
        // hands it on; after 32 steps lane l holds the warp's whole sum for
        // pair (l + 1) mod 32 of each group (fixed order: lane p first).
        const int ng = (min(kAdjRP, (re - r0 + 1) >> 1) + 31) >> 5;  // groups holding a valid pair
        float2 gz[kAdjGroups][3];
#pragma unroll
        for (int g2 = 0; g2 < kAdjGroups; ++g2)
#pragma unroll
          for (int a = 0; a < 3; ++a) gz[g2][a] = make_float2(0.f, 0.f);
        const int from = (lane + 31) & 31;
#pragma unroll 1
        for (int st = 0; st < 32; ++st) {
          if (st > 0) {
#pragma unroll
            for (int g2 = 0; g2 < kAdjGroups; ++g2)
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                gz[g2][a].x = __shfl_sync(0xffffffffu, gz[g2][a].x, from);
                gz[g2][a].y = __shfl_sync(0xffffffffu, gz[g2][a].y, from);
              }
          }
          const int pl = (lane - st) & 31;
#pragma unroll
          for (int g2 = 0; g2 < kAdjGroups; ++g2) {
            if (g2 >= ng) break;  // warp-uniform: a ragged chunk's empty groups
            const float4* rp = reinterpret_cast<const float4*>(&sm.rec[buf][g2 * 32 + pl][0]);
            const float4 a0 = rp[0], a1 = rp[1], a2 = rp[2], a3 = rp[3], a4 = rp[4], a5 = rp[5];
            const float2 nz0 = make_float2(a0.x, a0.y), nz1 = make_float2(a0.z, a0.w);
            const float2 nz2 = make_float2(a1.x, a1.y), ngA = make_float2(a1.z, a1.w);
            const float2 ngB0 = make_float2(a2.x, a2.y), ngB1 = make_float2(a2.z, a2.w);
            const float2 ngB2 = make_float2(a3.x, a3.y), ngC = make_float2(a3.z, a3.w);
            const float2 gB0 = make_float2(a4.x, a4.y), gB1 = make_float2(a4.z, a4.w);
            const float2 gB2 = make_float2(a5.x, a5.y);
            float2 gz0 = gz[g2][0], gz1 = gz[g2][1], gz2 = gz[g2][2];  // sum of e gB - w (x - z)
#pragma unroll
            for (int j = 0; j < kAdjCols; ++j) {
              const float2 dx = __fadd2_rn(xd[j][0], nz0);
              const float2 dy = __fadd2_rn(xd[j][1], nz1);
              const float2 dz = __fadd2_rn(xd[j][2], nz2);
              float2 d2 = __fmul2_rn(dx, dx);
              d2 = __ffma2_rn(dy, dy, d2);
              d2 = __ffma2_rn(dz, dz, d2);
              const float2 e = ex2_neg_pair(d2);
              float2 nge = __ffma2_rn(ngB0, xd[j][0], ngA);
              nge = __ffma2_rn(ngB1, xd[j][1], nge);
              nge = __ffma2_rn(ngB2, xd[j][2], nge);
              nge = __ffma2_rn(ngC, e, nge);
              // e (gB - ge (x - z) / s2): the column's term, and the row's
              // plus e gB (removed once per row at its completion)
              const float2 t0 = __ffma2_rn(nge, dx, gB0);
              const float2 t1 = __ffma2_rn(nge, dy, gB1);
              const float2 t2 = __ffma2_rn(nge, dz, gB2);
              gz0 = __ffma2_rn(e, t0, gz0);
              gz1 = __ffma2_rn(e, t1, gz1);
              gz2 = __ffma2_rn(e, t2, gz2);
              gx[j][0] = __ffma2_rn(e, t0, gx[j][0]);
              gx[j][1] = __ffma2_rn(e, t1, gx[j][1]);
              gx[j][2] = __ffma2_rn(e, t2, gx[j][2]);
            }
            gz[g2][0] = gz0;
            gz[g2][1] = gz1;
            gz[g2][2] = gz2;
          }
        }
        {
          const int pw = (lane + 1) & 31;  // the pair whose sum this lane holds
#pragma unroll
          for (int g2 = 0; g2 < kAdjGroups; ++g2) {
            if (g2 >= ng) break;
            const int row = 2 * (g2 * 32 + pw);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              sm.wsum[buf][a][warp][row] = gz[g2][a].x;
              sm.wsum[buf][a][warp][row + 1] = gz[g2][a].y;
            }
          }
        }
      }
      // the unit's last chunk: its row totals are complete after this barrier
      __syncthreads();
      {
        const int rl = rb + ((re - rb - 1) / kAdjRows) * kAdjRows;  // the last chunk's first row
        complete_chunk_rows(sm, buf ^ 1, rl + tid, re, cb, inv_sc, A);
      }
      // this unit's dL/dx of the owned columns
#pragma unroll
      for (int j = 0; j < kAdjCols; ++j) {
        const int c = cb * kAdjColBlk + j * kThreads + tid;
        if (c < A.N && px_dst)
          __stcg(px_dst + j * kThreads + tid,
                 make_float4((gx[j][0].x + gx[j][0].y) * inv_sc, (gx[j][1].x + gx[j][1].y) * inv_sc,
                             (gx[j][2].x + gx[j][2].y) * inv_sc, 0.f));
      }
    }
    if (tid == 0 && s_pair[0] >= 0)
      A.pair_t[2 * s_pair[0] + (s_pair[1] ^ s_pair[2])] = (float)(global_ns() - s_tsweep);
    if (!ok || !grid_sync(A.ctl, epoch, G, A.timeout_ns, 102)) {
      ok = false;
      break;
    }
    if (tid == 0 && s_pair[0] >= 0) {  // both blocks of the pair read the same two times
      long lo = 0, sp = 0, hi = 0;
      if (g.pair_num) {
        ranged_tasks(adj_tasks(g), 2 * s_pair[0], (int)G, lo, sp);
        ranged_tasks(adj_tasks(g), 2 * s_pair[0] + 1, (int)G, sp, hi);
      } else {
        const PairUnits pu = pair_units(g.units, (int)G / 2, s_pair[0]);
        lo = pu.lo;
        sp = pu.split;
        hi = pu.hi;
      }
      if (pair_swap(lo, sp, hi, A.pair_t, s_pair[0])) {
        s_pair[2] ^= 1;
        if (g.pair_num) rsh = ranged_share(adj_tasks(g), 2 * s_pair[0] + (s_pair[1] ^ s_pair[2]), (int)G);
      }
    }
    // Rows completed, each block a contiguous share of them (all blocks in
    // parallel, no serial tail): the column blocks' dL/dz partials summed in
    // column-block order, dL/dy = R^T dL/dz + lambda_r gP + gQ^T u_r, and the
    // block's record of sum dL/dz y^T (row-major, as R), sum dL/dz and, for
    // rows on the C_r <= 1e-6 branch (lambda = 1, u = mean X), sum gu_r.
    {
      const int rpc = (A.M + (int)G - 1) / (int)G;
      const int r0 = (int)blockIdx.x * rpc;
      const int nrows = max(0, min(rpc, A.M - r0));
      df vv[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) vv[q] = df_make(0.f);
      for (int r = r0 + tid; r < r0 + nrows; r += kThreads) {
        float totz[3] = {0.f, 0.f, 0.f};
        int b = 0;
        for (; b + 8 <= g.nb; b += 8) {  // 8 loads in flight, added in column-block order
          float4 pz[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) pz[j] = __ldcg(A.part_z + (size_t)(b + j) * A.M + r);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            totz[0] += pz[j].x;
            totz[1] += pz[j].y;
            totz[2] += pz[j].z;
          }
        }
        for (; b < g.nb; ++b) {
          const float4 pz = __ldcg(A.part_z + (size_t)b * A.M + r);
          totz[0] += pz.x;
          totz[1] += pz.y;
          totz[2] += pz.z;
        }
        const float4 y = ld_cg(A.rows + r);
        const float* rt = rtape + (size_t)r * 5;
        const float C = rt[0], lam = rt[1];
        const float uu[3] = {rt[2], rt[3], rt[4]};
        const float yy[3] = {y.x, y.y, y.z};
        float gu[3];
        for (int i = 0; i < 3; ++i)
          gu[i] = coef[1 + i] + coef[7 + i] * yy[0] + coef[10 + i] * yy[1] + coef[13 + i] * yy[2];
        // the sweep summed e (gB - w (x - z)) over the columns: its e gB part,
        // gB sum_c e = gu C^-1/2 A = gu lambda, comes off here
        if (C > 10e-7f)
          for (int i = 0; i < 3; ++i) totz[i] = fmaf(lam, gu[i], totz[i]);
        float gy[3];
        for (int jj = 0; jj < 3; ++jj)
          gy[jj] = R[jj] * totz[0] + R[3 + jj] * totz[1] + R[6 + jj] * totz[2] + lam * coef[4 + jj] +
                   coef[7 + 3 * jj] * uu[0] + coef[8 + 3 * jj] * uu[1] + coef[9 + 3 * jj] * uu[2];
        float4 o = A.gY[r];
        o.x += gy[0];
        o.y += gy[1];
        o.z += gy[2];
        A.gY[r] = o;
        for (int i = 0; i < 3; ++i) {
          for (int jj = 0; jj < 3; ++jj) df_add_prod(vv[3 * i + jj], totz[i], yy[jj]);  // dL/dR_ij, row-major
          df_add(vv[9 + i], totz[i]);
        }
        if (!(C > 10e-7f)) {  // branch rows: u = mean X
          for (int i = 0; i < 3; ++i) df_add(vv[12 + i], gu[i]);
        }
      }
      // the block's 16 sums, through shared memory (scr and wsum are free here)
      static_assert(sizeof(sm.wsum) >= sizeof(df) * 17 * kThreads, "moment scratch");
      em_block_moments(vv, min(kThreads, nrows), reinterpret_cast<df*>(&sm.wsum[0][0][0][0]),
                       recs + (size_t)blockIdx.x * 16);
    }
    if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, 103)) {
      ok = false;
      break;
    }
    // upstream gradient of the previous step's output pose, identical in every block
    reduce_block_partials<16>(recs, (int)G, s_red, s_tot);
    if (tid < 12) s_g[tid] = df_val(s_tot[tid]);
    __syncthreads();
    const float gxb[3] = {df_val(s_tot[12]) / (float)A.N, df_val(s_tot[13]) / (float)A.N,
                          df_val(s_tot[14]) / (float)A.N};
    // dL/dx_c: this block's share of the columns, the row-slice (ranged: the
    // kmax slot) partials in order
    for (int c = blockIdx.x * kThreads + tid; c < A.N; c += G * kThreads) {
      float sx = gxb[0], sy = gxb[1], sz = gxb[2];
      const int cbk = c / kAdjColBlk;
      const float4* src = g.ranged ? px + (size_t)cbk * g.kmax * kAdjColBlk + (c - cbk * kAdjColBlk) : px + c;
      const size_t stride = g.ranged ? (size_t)kAdjColBlk : (size_t)A.N;
      const int np = g.ranged ? g.kmax : g.S;
      int b = 0;
      for (; b + 16 <= np; b += 16) {  // 16 loads in flight, summed in order
        float4 p[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) p[j] = __ldcg(src + (size_t)(b + j) * stride);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          sx += p[j].x;
          sy += p[j].y;
          sz += p[j].z;
        }
      }
      for (; b < np; ++b) {
        const float4 p = __ldcg(src + (size_t)b * stride);
        sx += p.x;
        sy += p.y;
        sz += p.z;
      }
      float4 o = A.gX[c];
      o.x += sx;
      o.y += sy;
      o.z += sz;
      A.gX[c] = o;
    }
  }
  if (blockIdx.x == 0 && tid == 0) {
    const int st = ld_status(A.ctl);
    if (st == kStatusOk) {
      // centred frame -> caller frame: t' = t + R oY - oX
      for (int i = 0; i < 3; ++i) {
        A.g_in[9 + i] = s_g[9 + i];
        for (int j = 0; j < 3; ++j) A.g_in[3 * i + j] = s_g[3 * i + j] + s_g[9 + i] * A.hdr->oY[j];
      }
    }
    if (A.d_status) *A.d_status = st;
  }
}

// float4 accumulators -> caller SoA [x..., y..., z...]
__global__ void adjoint_unpack_kernel(const float4* gX, int N, float* oX, const float4* gY, int M, float* oY) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) {
    const float4 v = gX[i];
    oX[i] = v.x;
    oX[N + i] = v.y;
    oX[2 * N + i] = v.z;
  } else if (i < N + M) {
    const int r = i - N;
    const float4 v = gY[r];
    oY[r] = v.x;
    oY[M + r] = v.y;
    oY[2 * M + r] = v.z;
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

struct AdjPlan {
  int grid;
  AdjGeom geo;
  size_t smem;
  int pairs;  // slice units dealt to SM pairs
};

// Column blocks of kAdjColBlk columns and row slices of an even number of rows,
// as many slices as fill whole waves of the co-resident grid best (up to 4 waves;
// at least 64 rows per slice).
AdjPlan plan_adj(int N, int M, int device, int layout) {
  AdjPlan P;
  P.smem = sizeof(AdjSmem);
  const int limit = persistent_grid_limit(device, (const void*)emicp_adjoint_kernel, P.smem);
  AdjGeom g;
  g.nb = (N + kAdjColBlk - 1) / kAdjColBlk;
  const int max_s = (M + 63) / 64;  // at least 64 rows per slice
  int bestS = 1;
  double best = -1.0;
#ifndef CESA_ADJ_MAX_WAVES
#define CESA_ADJ_MAX_WAVES 4
#endif
  for (int w = 1; w <= CESA_ADJ_MAX_WAVES; ++w) {
    int S = (w * limit) / g.nb;
    if (S < 1) S = 1;
    if (S > max_s) S = max_s;
    const int units = g.nb * S;
    const int waves = (units + limit - 1) / limit;
    const double eff = (double)units / ((double)waves * limit);
    if (eff > best + 0.02) {
      best = eff;
      bestS = S;
    }
  }
  g.len = (M + bestS - 1) / bestS;
  g.len += g.len & 1;
  g.S = (M + g.len - 1) / g.len;
  g.units = g.nb * g.S;
  g.ranged = 0;
  g.nch = (M + kAdjRows - 1) / kAdjRows;
  g.kmax = 0;
  g.pair_num = 0;
  P.geo = g;
  P.grid = g.units < limit ? g.units : limit;
  // SM pairs (two blocks on every SM): slice units dealt to pairs (at least
  // four units per pair), or the ranged tasks split within each pair
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const char* ev = getenv("CESA_SM_PAIRS");  // "0": equal shares (for comparisons)
  const bool two_per_sm = sms > 0 && limit == 2 * sms && !(ev && ev[0] == '0');
  // AUTO: ranged tasks for large clouds when SM pairs split them (the split
  // is then finer than whole units), else where their longest run (in
  // 256-row chunks) is shorter than the slice plan's (its waves times the
  // chunks of a slice).
  const long T = (long)g.nb * g.nch;
  const long per = (T + limit - 1) / limit;
  const int waves = (g.units + limit - 1) / limit;
  const bool ranged =
      layout == CESA_LAYOUT_RANGED ||
      (layout == CESA_LAYOUT_AUTO && T >= 8L * limit &&
       (two_per_sm || (double)per < (double)waves * g.len / kAdjRows));
  if (ranged) {
    P.geo.ranged = 1;
    P.geo.pair_num = two_per_sm ? kAdjRangedPairNum : 0;
    P.geo.kmax = ranged_kmax(adj_tasks(P.geo), limit);  // tasks of kAdjRows rows: g.nch as set above
    P.grid = limit;
  }
  P.pairs = !P.geo.ranged && two_per_sm && P.grid == limit && P.geo.units >= 2 * P.grid;
  return P;
}

// float4s of the dL/dx partials, both step parities
size_t part_x_len(const AdjGeom& g, int N) {
  return g.ranged ? (size_t)2 * g.nb * g.kmax * kAdjColBlk : (size_t)2 * g.S * N;
}

}  // namespace

// Workspace of the adjoint: control block and counters (cleared), gradient
// accumulators gX, gY (cleared), split partials, records and column partials.
size_t emicp_adjoint_ws_need(int N, int M, int device, int layout) {
  const AdjPlan P = plan_adj(N, M, device, layout);
  Carve c(nullptr);
  c.take<Ctl>(1);
  c.take<float4>((size_t)N);
  c.take<float4>((size_t)M);
  c.take<float>(12);
  c.take<unsigned>(2 * kPairCap + 1);
  c.take<float>((size_t)P.grid);
  c.take<float4>((size_t)P.geo.nb * M);
  c.take<df>((size_t)2 * P.grid * 16);
  c.take<float4>(part_x_len(P.geo, N));
  return c.off;
}

int enqueue_emicp_adjoint(const EmicpAdjointLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  const AdjPlan P = plan_adj(L.N, L.M, device, L.layout);
  Carve c(ws);
  Ctl* ctl = c.take<Ctl>(1);
  float4* gX = c.take<float4>((size_t)L.N);
  float4* gY = c.take<float4>((size_t)L.M);
  float* g_in = c.take<float>(12);
  unsigned* pair_tab = c.take<unsigned>(2 * kPairCap + 1);
  const size_t zero_bytes = c.off;
  float* pair_t = c.take<float>((size_t)P.grid);
  float4* part_z = c.take<float4>((size_t)P.geo.nb * L.M);
  df* rec = c.take<df>((size_t)2 * P.grid * 16);
  float4* part_x = c.take<float4>(part_x_len(P.geo, L.N));
  if (c.off > ws_bytes) return (int)cudaErrorInvalidValue;
  e = cudaMemsetAsync(ws, 0, zero_bytes, st);
  // ranged dL/dx slots that no block writes must read as zero
  if (e == cudaSuccess && P.geo.ranged) e = cudaMemsetAsync(part_x, 0, sizeof(float4) * part_x_len(P.geo, L.N), st);
  if (e != cudaSuccess) return (int)e;
  EmAdjArgs A;
  A.rows = L.rows;
  A.cols = L.cols;
  A.M = L.M;
  A.N = L.N;
  A.geo = P.geo;
  A.nsteps = L.nsteps;
  A.tape = L.tape;
  A.row_tape = L.row_tape;
  A.g_out = L.g_out;
  A.hdr = L.hdr;
  A.gX = gX;
  A.gY = gY;
  A.g_in = g_in;
  A.part_z = part_z;
  A.rec = rec;
  A.part_x = part_x;
  A.ctl = ctl;
  A.pair_tab = pair_tab;
  A.pair_t = pair_t;
  A.pairs = P.pairs;
  A.d_status = L.d_status;
  A.timeout_ns = L.timeout_ns;
  if (L.nsteps > 0) {
    void* args[] = {(void*)&A};
    e = cudaLaunchCooperativeKernel((const void*)emicp_adjoint_kernel, dim3(P.grid), dim3(kThreads), args, P.smem,
                                    st);
    if (e != cudaSuccess) return (int)e;
  } else {
    e = cudaMemcpyAsync(g_in, L.g_out, sizeof(float) * 12, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return (int)e;
  }
  // SoA outputs
  adjoint_unpack_kernel<<<(L.N + L.M + 255) / 256, 256, 0, st>>>(gX, L.N, L.gX, gY, L.M, L.gY);
  if (e == cudaSuccess) e = cudaMemcpyAsync(L.g_in, g_in, sizeof(float) * 12, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  return (int)e;
}

}  // namespace cesa
