// Per-element functors, row finalizers and moment assembly shared by the
// single-pair and the batched registration kernels (sm_103a).
#pragma once
#include "cesa_sweep.cuh"

namespace cesa {

// Element functors work on two owned points at once with packed FP32 pairs
// (FFMA2/FADD2/FMUL2 on sm_100+: the same round-to-nearest operations as the
// scalar code, so results are unchanged, at half the issued instructions).
// q holds the negated coordinates of the two owned points; s is the streamed
// point and h its second record.
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// Squared distances |s - p|^2 of one streamed point to two owned points:
// 3 FADD, FMUL + 2 FFMA each, as direct differences.
__device__ __forceinline__ float2 dist2_pair(const float2 (&q)[3], float4 s) {
  const float2 dx = __fadd2_rn(dup2(s.x), q[0]);
  const float2 dy = __fadd2_rn(dup2(s.y), q[1]);
  const float2 dz = __fadd2_rn(dup2(s.z), q[2]);
  float2 d2 = __fmul2_rn(dx, dx);
  d2 = __ffma2_rn(dy, dy, d2);
  return __ffma2_rn(dz, dz, d2);
}

__device__ __forceinline__ float2 ex2_pair(float2 t) { return make_float2(ex2_approx(t.x), ex2_approx(t.y)); }

// 2^-t of a packed pair (the negation is the exponential's operand, not a
// separate instruction).
__device__ __forceinline__ float2 ex2_neg_pair(float2 t) { return make_float2(ex2_approx(-t.x), ex2_approx(-t.y)); }

// ------------------------------------------------------------------ EM-ICP
constexpr int kEmNV = 16;  // moments: sum lambda, sum u (3), sum lambda y (3), sum u y^T (9)

// Per-element work of the fused one-pass E-step, with e = exp(-d^2 / (2 sigma_p2)):
// running sums of e^2, e and e x over the streamed X points of one owned Y row.
struct EmicpElem {
  float nk;  // -log2(e) / (2 sigma_p2)
  __device__ __forceinline__ void operator()(float2 (&acc)[5], const float2 (&q)[3], float4 x, float4) const {
    const float2 e = ex2_pair(__fmul2_rn(dist2_pair(q, x), dup2(nk)));
    acc[0] = __ffma2_rn(e, e, acc[0]);
    acc[1] = __fadd2_rn(acc[1], e);
    acc[2] = __ffma2_rn(e, dup2(x.x), acc[2]);
    acc[3] = __ffma2_rn(e, dup2(x.y), acc[3]);
    acc[4] = __ffma2_rn(e, dup2(x.z), acc[4]);
  }
};

// The same with both clouds scaled by sc = sqrt(log2(e) / (2 sigma_p2)) (the
// streamed X' and the owned R y + t): e = 2^-|x' - z'|^2, one packed multiply
// fewer per pair; the e x sums come out sc times too large.
struct EmicpElemScaled {
  __device__ __forceinline__ void operator()(float2 (&acc)[5], const float2 (&q)[3], float4 x, float4) const {
    const float2 e = ex2_neg_pair(dist2_pair(q, x));
    acc[0] = __ffma2_rn(e, e, acc[0]);
    acc[1] = __fadd2_rn(acc[1], e);
    acc[2] = __ffma2_rn(e, dup2(x.x), acc[2]);
    acc[3] = __ffma2_rn(e, dup2(x.y), acc[3]);
    acc[4] = __ffma2_rn(e, dup2(x.z), acc[4]);
  }
};

// One row's finalize: from its sums tot = (sum e^2, sum e, sum e x) to C_r,
// lambda_r, u_r = lambda_r X'_r (src/emicp.cu:489-549: C_r <= 1e-6 gives
// A = 1/N, lambda = 1, X' = mean(X)), the optional row records, and the row's
// contribution to the 16 moments (added to v).
__device__ __forceinline__ void emicp_row_finish(int r, const float (&tot)[5], float4 y, float outlier,
                                                 const float (&xm)[3], float* row_out, const float (&oX)[3],
                                                 float* row_tape, df (&v)[kEmNV]) {
  const float C = tot[0] + outlier;
  float lam, uu[3];
  if (C > 10e-7f) {  // src/emicp.cu:155
    const float inv = __frsqrt_rn(C);
    lam = tot[1] * inv;
    uu[0] = tot[2] * inv;
    uu[1] = tot[3] * inv;
    uu[2] = tot[4] * inv;
  } else {  // A <- 1/N (src/emicp.cu:159): lambda = 1, lambda X' = mean(X)
    lam = 1.f;
    uu[0] = xm[0];
    uu[1] = xm[1];
    uu[2] = xm[2];
  }
  if (row_tape) {
    float* o = row_tape + (size_t)r * 5;
    o[0] = C;
    o[1] = lam;
    o[2] = uu[0];
    o[3] = uu[1];
    o[4] = uu[2];
  }
  if (row_out) {
    float* o = row_out + (size_t)r * 5;
    o[0] = C;
    o[1] = lam;
    o[2] = fmaf(lam, oX[0], uu[0]);
    o[3] = fmaf(lam, oX[1], uu[1]);
    o[4] = fmaf(lam, oX[2], uu[2]);
  }
  const float yy[3] = {y.x, y.y, y.z};
  df_add(v[0], lam);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    df_add(v[1 + i], uu[i]);
    df_add_prod(v[4 + i], lam, yy[i]);
  }
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) df_add_prod(v[7 + i + 3 * j], uu[i], yy[j]);
}

// Row finalize of a split-completed owned block (the batched kernel): every
// row's emicp_row_finish, then the block's 16 moments (block accumulator,
// compensated).
struct EmicpFin {
  const float4* rows;
  int M;
  float outlier;
  float xm[3];
  float* row_out;  // caller frame: u = lambda X' + lambda oX
  float oX[3];
  df* scratch;     // shared, >= 17 * 128 dfs
  df* rbpart;      // this step's [nblk][kEmNV]
  float* row_tape; // optional: this step's [M][5] (C, lambda, u) in the centred frame
  __device__ void operator()(int blk, const float (&tot)[5]) const {
    df v[kEmNV];
#pragma unroll
    for (int k = 0; k < kEmNV; ++k) v[k] = df_make(0.f);
    const int r = blk * kBlockPts + (int)threadIdx.x;
    if (threadIdx.x < kBlockPts && r < M)
      emicp_row_finish(r, tot, ld_cg(rows + r), outlier, xm, row_out, oX, row_tape, v);
    owned_block_sum<kEmNV>(v, scratch, rbpart + (size_t)blk * kEmNV);
  }
};

// Sum over the block of the 16 moments held by threads 0..active-1 (active <=
// kThreads), through shared memory in a fixed order: value k of thread i at
// scratch[k * kThreads + i]; thread (k, g) = (tid % 16, tid / 16) adds entries
// g, g + 16, ...; thread k adds the 16 group sums. The record goes to dst.
__device__ __forceinline__ void em_block_moments(const df (&v)[kEmNV], int active, df* scratch, df* dst) {
  static_assert(kEmNV == 16 && kThreads % 16 == 0, "16 moments");
  const int tid = threadIdx.x;
  df* part = scratch + kEmNV * kThreads;
  if (tid < active)
#pragma unroll
    for (int k = 0; k < kEmNV; ++k) scratch[k * kThreads + tid] = v[k];
  __syncthreads();
  if (active <= kThreads / kEmNV) {
    // one entry per group: thread k adds the active threads' values in order,
    // bitwise what the two-level sum gives (its other terms are zeros)
    if (tid < kEmNV) {
      df s = df_make(0.f);
      for (int i = 0; i < active; ++i) df_add(s, scratch[tid * kThreads + i]);
      __stcg(reinterpret_cast<float2*>(dst + tid), make_float2(s.hi, s.lo));
    }
    __syncthreads();
    return;
  }
  {
    const int k = tid % kEmNV, g = tid / kEmNV;
    df s = df_make(0.f);
    for (int i = g; i < active; i += kThreads / kEmNV) df_add(s, scratch[k * kThreads + i]);
    part[k * (kThreads / kEmNV) + g] = s;
  }
  __syncthreads();
  if (tid < kEmNV) {
    df s = part[tid * (kThreads / kEmNV)];
#pragma unroll
    for (int g = 1; g < kThreads / kEmNV; ++g) df_add(s, part[tid * (kThreads / kEmNV) + g]);
    __stcg(reinterpret_cast<float2*>(dst + tid), make_float2(s.hi, s.lo));
  }
  __syncthreads();
}

__device__ __forceinline__ df dmul(df a, float b) {  // (a.hi + a.lo) * b, ~df precision
  df r = df_make(0.f);
  df_add_prod(r, a.hi, b);
  r.lo = __fmaf_rn(a.lo, b, r.lo);
  return r;
}
__device__ __forceinline__ df dsub(df a, const df& b) {
  df_add(a, df{-b.hi, -b.lo});
  return a;
}

// Centres and cross-covariance from the 16 EM-ICP moments (centred frame):
// Xc = sum u / L, Yc = sum lambda y / L and
//   S = sum u y^T - Xc (sum lambda y)^T - (sum u) Yc^T + L Xc Yc^T,
// the expansion of sum (u - lambda Xc)(y - Yc)^T (src/emicp.cu's centring of
// X' and Y before the product), every product in df. With the FP32-rounded
// centres the first-order rounding terms cancel and L dXc dYc^T remains, so a
// cloud that sits off the origin (raw moments thousands of times S) keeps S
// to FP32 precision; S = sum u y^T - L Xc Yc^T with rounded Xc would not.
__device__ __forceinline__ float em_S_entry(const df* tot, int i, int j, float xi, float yj) {
  df a = tot[7 + i + 3 * j];
  df_add(a, dmul(tot[4 + j], -xi));
  df_add(a, dmul(tot[1 + i], -yj));
  df_add(a, dmul(dmul(tot[0], xi), yj));
  return df_val(a);
}

// One thread forms everything (the adjoint's recomputation of a step).
__device__ __forceinline__ void em_moments_to_S(const df* tot, float Xc[3], float Yc[3], float S[9]) {
  const float L = df_val(tot[0]);
  for (int i = 0; i < 3; ++i) {
    Xc[i] = df_val(tot[1 + i]) / L;
    Yc[i] = df_val(tot[4 + i]) / L;
  }
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) S[i + 3 * j] = em_S_entry(tot, i, j, Xc[i], Yc[j]);
}

// Block-wide (every thread calls it), bitwise the same values: thread i + 3 j
// (< 9) forms S_ij, threads 9..14 the centres, into out[0..8] = S,
// out[9..11] = Xc, out[12..14] = Yc (shared). The nine df chains then run side
// by side instead of one after another in one thread. Synchronises the block.
__device__ __forceinline__ void em_moments_to_S_block(const df* tot, float* out) {
  const int t = threadIdx.x;
  if (t < 15) {
    const float L = df_val(tot[0]);
    if (t < 9) {
      const int i = t % 3, j = t / 3;
      out[t] = em_S_entry(tot, i, j, df_val(tot[1 + i]) / L, df_val(tot[4 + j]) / L);
    } else {
      out[t] = df_val(tot[t - 8]) / L;  // t = 9..11: tot[1..3] (Xc); 12..14: tot[4..6] (Yc)
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------ Softassign
constexpr int kSaNV = 32;

// Sinkhorn sweep element: acc += K * weight(streamed).
struct SinkElem {
  float nk, c0;  // K = 2^(c0 + nk d^2)
  __device__ __forceinline__ void operator()(float2 (&acc)[1], const float2 (&q)[3], float4 s, float4) const {
    const float2 e = ex2_pair(__ffma2_rn(dist2_pair(q, s), dup2(nk), dup2(c0)));
    acc[0] = __ffma2_rn(e, dup2(s.w), acc[0]);
  }
};

// The same with both clouds scaled by sc = sqrt(log2(e) / T) and 2^c0 folded
// into the streamed weight (w = 2^c0 b): K / 2^c0 = 2^-|x' - y'|^2, one packed
// op fewer per pair.
struct SinkElemScaled {
  __device__ __forceinline__ void operator()(float2 (&acc)[1], const float2 (&q)[3], float4 s, float4) const {
    const float2 e = ex2_neg_pair(dist2_pair(q, s));
    acc[0] = __ffma2_rn(e, dup2(s.w), acc[0]);
  }
};

// Final row sweep element: w += K b, mu += K delta, Vhat += K g (y' - Yhat).
struct FinalElem {
  float nk, c0;
  __device__ __forceinline__ void operator()(float2 (&acc)[5], const float2 (&q)[3], float4 s, float4 h) const {
    const float2 e = ex2_pair(__ffma2_rn(dist2_pair(q, s), dup2(nk), dup2(c0)));
    acc[0] = __ffma2_rn(e, dup2(s.w), acc[0]);
    acc[1] = __ffma2_rn(e, dup2(h.w), acc[1]);
    acc[2] = __ffma2_rn(e, dup2(h.x), acc[2]);
    acc[3] = __ffma2_rn(e, dup2(h.y), acc[3]);
    acc[4] = __ffma2_rn(e, dup2(h.z), acc[4]);
  }
};

// The final sweep element on scaled clouds, with 2^c0 folded into the four
// streamed weights (b, delta, g (y' - Yhat)), as in SinkElemScaled.
struct FinalElemScaled {
  __device__ __forceinline__ void operator()(float2 (&acc)[5], const float2 (&q)[3], float4 s, float4 h) const {
    const float2 e = ex2_neg_pair(dist2_pair(q, s));
    acc[0] = __ffma2_rn(e, dup2(s.w), acc[0]);
    acc[1] = __ffma2_rn(e, dup2(h.w), acc[1]);
    acc[2] = __ffma2_rn(e, dup2(h.x), acc[2]);
    acc[3] = __ffma2_rn(e, dup2(h.y), acc[3]);
    acc[4] = __ffma2_rn(e, dup2(h.z), acc[4]);
  }
};

// Final row finalize: w, mu = m - w, Vhat (times a_r) and the 28 row-side moments.
//  0: sum w            1-3: sum w x'         4-12: sum w x'_i Vhat_j (i + 3j)
// 13-15: sum Vhat       16-18: sum w mu x'    19: sum mu
// 20-22: sum w^2 x'     23: sum w^2           24-26: sum w Vhat      27: sum w mu
// One row's contribution to the 28 row-side moments (slots as listed above).
template <int NV>
__device__ __forceinline__ void sa_row_moments(df (&v)[NV], float w, float mu, const float (&V)[3],
                                               const float (&xp)[3]) {
  static_assert(NV >= 28, "28 row moments");
  const float w2 = w * w, wmu = w * mu;
  df_add(v[0], w);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    df_add_prod(v[1 + i], w, xp[i]);
    const float wx = w * xp[i];
#pragma unroll
    for (int j = 0; j < 3; ++j) df_add_prod(v[4 + i + 3 * j], wx, V[j]);
    df_add(v[13 + i], V[i]);
    df_add_prod(v[16 + i], wmu, xp[i]);
    df_add_prod(v[20 + i], w2, xp[i]);
    df_add_prod(v[24 + i], w, V[i]);
  }
  df_add(v[19], mu);
  df_add_prod(v[23], w, w);
  df_add_prod(v[27], w, mu);
}

struct FinalFin {
  const float4* rows;
  const float* a;  // a^(I1)
  float* w_out;
  int N;
  df* scratch;     // shared, >= 33 * 128 dfs
  df* rbpart;      // this update's row-block records [nblk_r][32] (slots 0..27 used)
  float* tape_fin = nullptr;  // optional [5][N]: the raw row sums tot[]
  __device__ void operator()(int blk, const float (&tot)[5]) const {
    df v[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = df_make(0.f);
    const int r = blk * kBlockPts + (int)threadIdx.x;
    if (threadIdx.x < kBlockPts && r < N) {
      const float4 x = __ldcg(&rows[r]);
      const float ar = __ldcg(a + r);
      const float w = ar * tot[0], mu = ar * tot[1];
      const float V[3] = {ar * tot[2], ar * tot[3], ar * tot[4]};
      const float xp[3] = {x.x, x.y, x.z};
      if (w_out) w_out[r] = w;
      if (tape_fin) {
#pragma unroll
        for (int m = 0; m < 5; ++m) __stcg(tape_fin + (size_t)m * N + r, tot[m]);
      }
      sa_row_moments(v, w, mu, V, xp);
    }
    owned_block_sum<32>(v, scratch, rbpart + (size_t)blk * 32);
  }
};

// df helpers for the moment assembly
// Softassign S and centres from the 32 moments, one value per thread
// (tid 0..8: S_ij, tid 9..11: centres). oX, oY: centring offsets; yh: mean(Y').
//   Yc = (B2 + oY B1)/A1, alpha = Yhat + oY, beta = alpha - Yc,
//   S_ij = (T1_ij - Xc'_i T3_j) + (T4_i - Xc'_i T5) alpha_j + (T6_i - Xc'_i A1) beta_j
//        + oX_i (T8_j - T3_j) + (T9 - T5) oX_i alpha_j + (T7 - A1) oX_i beta_j
__device__ __forceinline__ void sa_moments_to_S(int tid, const df* s_tot, const float* oX, const float* oY,
                                                const float* yh, float* s_S, float* s_xcp, float* s_yd,
                                                float* s_xc, float* s_yc) {
  const df A1 = s_tot[0];
  const float inv = 1.f / df_val(A1);
  const float rho = df_val(s_tot[28]) * inv;
  if (tid < 9) {
    const int i = tid % 3, j = tid / 3;
    const float xi = df_val(s_tot[1 + i]) * inv;
    const float al = yh[j] + oY[j];
    df bj = df_make(yh[j]);  // beta_j = (Yhat_j - B2_j/A1) - (rho - 1) oY_j
    df_add(bj, -df_val(s_tot[29 + j]) * inv);
    df_add_prod(bj, 1.f - rho, oY[j]);
    const float be = df_val(bj);
    const df T5 = s_tot[19], T7 = s_tot[23], T9 = s_tot[27];
    df P2 = s_tot[16 + i];
    df_add(P2, dmul(T5, -xi));
    df P3 = s_tot[20 + i];
    df_add(P3, dmul(A1, -xi));
    df sij = s_tot[4 + i + 3 * j];
    df_add(sij, dmul(s_tot[13 + j], -xi));
    df_add(sij, dmul(P2, al));
    df_add(sij, dmul(P3, be));
    df_add(sij, dmul(dsub(s_tot[24 + j], s_tot[13 + j]), oX[i]));
    df_add(sij, dmul(dsub(T9, T5), oX[i] * al));
    df_add(sij, dmul(dsub(T7, A1), oX[i] * be));
    s_S[i + 3 * j] = df_val(sij);
  } else {
    const int i = tid - 9;
    const float xi = df_val(s_tot[1 + i]) * inv;
    s_xcp[i] = xi;
    s_xc[i] = xi + oX[i];
    df yd = df_make(df_val(s_tot[29 + i]) * inv);  // Yc - oY = B2/A1 + (rho - 1) oY
    df_add_prod(yd, rho - 1.f, oY[i]);
    s_yd[i] = df_val(yd);
    df yc = yd;
    df_add(yc, oY[i]);
    s_yc[i] = df_val(yc);
  }
}

}  // namespace cesa
