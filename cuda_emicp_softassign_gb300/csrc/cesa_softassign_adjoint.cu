// Adjoint of Softassign (src/softassign.cu:486-822) for sm_103a.
//
// One inner iteration (src/softassign.cu:494-798) maps (pose, s, u) to
// (pose', s', u') at temperature T for fixed X, Y. With
// K_ij = exp((alpha - |x_i - z_j|^2)/T)/sqrt(T), z_j = R y_j + t, a^0 = 1,
// b^0 = 1, s^0 = s, u^0 = u:
//   row pass k:    r^k = K b^k,       rs^k = a^k r^k + s^k,  a^{k+1} = a^k/rs^k,  s^{k+1} = s^k/rs^k
//   column pass k: c^k = K^T a^{k+1}, cs^k = b^k c^k + u^k,  b^{k+1} = b^k/cs^k,  u^{k+1} = u^k/cs^k
//   final:  rho = K b, w = a rho, sumM = sum w, Xc = sum w x / sumM,
//           Yc = sum cs y / sumM, p_i = w_i x_i - Xc, h_j = b_j (cs_j y_j - Yc),
//           V = K h, S = sum_i a_i p_i V_i^T, (R', t') = Horn(S, Xc, Yc)
// with a = a^{I1}, b = b^{I1}, cs = cs^{I1-1}, all in the caller's frame
// (the reference's S is not translation invariant). The forward kernel tapes
// every one of these vectors (the scalings and sums of each pass, the final
// sweep's row sums and Horn's solve; O(N + M) per pass), so the backward of
// an update runs no forward sweep: it applies the chain rule through Horn's
// pose (horn_pose_adjoint), the final stage, and the column and row passes in
// reverse. Each pass's adjoint is one K or K^T product (K recomputed, never
// stored). dL/dK is a sum of 4 + 2 I1 rank-1 terms alpha_m beta_m^T:
//   (g(V)_d, h_d) d = 0..2,  (g(rho), b^{I1}),  (a^{k+1}, g(c^k)),  (g(r^k), b^k)
// so dL/dx and dL/dz come from recomputing G = K .* dL/dK once more:
// dL/dx_i = (2/T) sum_j G_ij (z_j - x_i) and likewise for z. The per-update
// launches do it in one sweep that owns the rows and also sums each streamed
// column over its owned block (a transposed shared-memory sum); the
// persistent backward runs two sweeps (own rows, own columns), which keep its
// latency-bound small sizes free of the transposes. dL/dy = R^T dL/dz plus the
// direct terms of Yc and h;
// dL/dR, dL/dt of the input pose are sum dL/dz y^T and sum dL/dz.
// V_i = sum_j K_ij h_j comes from the final sweep's sums rho = K b,
// m = K (b (cs - 1)) and v = K (b cs (y' - Yhat)):
//   V = v + (Yhat - (Yc - oY)) rho + (Yhat + oY) m.
//
// Sweeps are plain launches over (owned block, streamed slice) tiles: each
// thread owns 4 points (two packed FP32 pairs) and the streamed points pass
// through shared memory. Slice partials are summed in slice order, so every
// result is deterministic. O(N + M) steps are small kernels; sums over all
// points use compensated arithmetic.
#include <cuda_runtime.h>

#include <algorithm>

#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {
namespace {

constexpr int kSwT = 128;                 // threads per sweep block
constexpr int kOwnBlk = kSwT * 4;         // owned points per sweep block (4 per thread)
constexpr int kTile = kSwT;               // streamed points per shared-memory tile
constexpr int kMaxTerms = 10;             // rank-1 terms per gradient sweep
constexpr int kGlue = 256;                // threads of the per-point kernels
// Threads of the one-block reductions (sums over all points): the block
// reduction's last step is serial over the warps, so small clouds use 8 warps
// and large ones 32 (where the per-thread point loop dominates).
constexpr int kOneBlock = 1024;
int one_block_threads(int n) { return n > 4096 ? 1024 : 256; }

struct Pose12 {
  float R[9], t[3];
};

__device__ __forceinline__ Pose12 load_pose(const float* p) {
  Pose12 P;
#pragma unroll
  for (int k = 0; k < 9; ++k) P.R[k] = __ldg(p + k);
#pragma unroll
  for (int k = 0; k < 3; ++k) P.t[k] = __ldg(p + 9 + k);
  return P;
}

__device__ __forceinline__ float4 posed(const Pose12& P, float4 y) {
  return make_float4(P.R[0] * y.x + P.R[1] * y.y + P.R[2] * y.z + P.t[0],
                     P.R[3] * y.x + P.R[4] * y.y + P.R[5] * y.z + P.t[1],
                     P.R[6] * y.x + P.R[7] * y.y + P.R[8] * y.z + P.t[2], 0.f);
}

// One sweep's geometry: the owned side (n_own points, optionally posed) and the
// streamed side, cut into S slices of len points.
struct SweepIO {
  const float4* own;
  const float4* str;
  int n_own, n_str;
  bool own_posed, str_posed;
  int S, len;
};

// Owned point of (thread, pair p, lane l) in owned block ob: coalesced per (p, l).
__device__ __forceinline__ int own_index(int ob, int p, int l) {
  return ob * kOwnBlk + (2 * p + l) * kSwT + (int)threadIdx.x;
}

// The lane's owned points, posed if the side is, negated and scaled by sc.
__device__ __forceinline__ void load_owned(const SweepIO& io, const Pose12& P, float sc, int ob, float2 (&q)[2][3]) {
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    float v[2][3];
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const int i = own_index(ob, p, l);
      float4 o = i < io.n_own ? io.own[i] : make_float4(0.f, 0.f, 0.f, 0.f);
      if (io.own_posed) o = posed(P, o);
      v[l][0] = -o.x * sc;
      v[l][1] = -o.y * sc;
      v[l][2] = -o.z * sc;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) q[p][d] = make_float2(v[0][d], v[1][d]);
  }
}

// The per-update record copy carries T and alpha in otherwise unused slots.
constexpr int kRecT = 60, kRecAlpha = 61;

// K = exp((alpha - d^2)/T)/sqrt(T) = 2^(c0 + nk d^2) = wsc 2^-|sc x - sc y|^2
// with sc = sqrt(-nk) and wsc = 2^c0, as the forward's matrix-free kernel forms
// it: the sweeps see the clouds scaled by sc and fold wsc into one side's
// weights, so an element needs no exponent op of its own.
__device__ __forceinline__ void kernel_consts(float T, float alpha, float& sc, float& wsc) {
  const float kk = kLog2e / T;
  sc = sqrtf(kk);
  wsc = exp2f(fmaf(alpha, kk, -0.5f * log2f(T)));
}

// Rank-1 terms of dL/dK: own side alpha, streamed side beta.
struct Terms {
  const float* own[kMaxTerms];
  const float* str[kMaxTerms];
  int n;
};

// Shared memory of one sweep tile (the streamed points and their weights).
struct SweepSmem {
  float4 pt[kTile];
  float w[kMaxTerms][kTile];
};

// One tile of a K product: part[sl][m][i] = sum over slice sl of
// K(own_i, str_j) w_m[j], m < NW, for the owned block ob (kSwT threads).
template <int NW>
__device__ __forceinline__ void sweep_sum_tile(const SweepIO& io, const Pose12& P, float sc, float wsc, const float* w,
                                               int ldw, float* part, int ob, int sl, SweepSmem& sm) {
  float2 q[2][3];
  load_owned(io, P, sc, ob, q);
  float2 acc[2][NW];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int m = 0; m < NW; ++m) acc[p][m] = make_float2(0.f, 0.f);
  const int jb = sl * io.len, je = min(jb + io.len, io.n_str);
  for (int j0 = jb; j0 < je; j0 += kTile) {
    const int n = min(kTile, je - j0);
    __syncthreads();
    if ((int)threadIdx.x < n) {
      const int j = j0 + threadIdx.x;
      float4 s = io.str[j];
      if (io.str_posed) s = posed(P, s);
      s = make_float4(s.x * sc, s.y * sc, s.z * sc, w[j] * wsc);
#pragma unroll
      for (int m = 1; m < NW; ++m) sm.w[m - 1][threadIdx.x] = w[(size_t)m * ldw + j] * wsc;
      sm.pt[threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll 8  // independent element chains (C5 backward 561 -> 544 ms over 2)
    for (int j = 0; j < n; ++j) {
      const float4 s = sm.pt[j];
      float wm[NW];
      wm[0] = s.w;
#pragma unroll
      for (int m = 1; m < NW; ++m) wm[m] = sm.w[m - 1][j];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const float2 e = ex2_neg_pair(dist2_pair(q[p], s));
#pragma unroll
        for (int m = 0; m < NW; ++m) acc[p][m] = __ffma2_rn(e, dup2(wm[m]), acc[p][m]);
      }
    }
  }
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const int i = own_index(ob, p, l);
      if (i < io.n_own)
#pragma unroll
        for (int m = 0; m < NW; ++m) part[((size_t)sl * NW + m) * io.n_own + i] = l ? acc[p][m].y : acc[p][m].x;
    }
}

// One tile of a gradient sweep: part[sl][d][i] = (2/T) sum over slice sl of
// G_ij (s_j - o_i)_d with G_ij = K_ij sum_m own_m[i] str_m[j].
__device__ __forceinline__ void sweep_grad_tile(const SweepIO& io, const Pose12& P, float sc, float wsc, float T,
                                                const Terms& tm, float* part, int ob, int sl, SweepSmem& sm) {
  float2 q[2][3];
  load_owned(io, P, sc, ob, q);
  float2 al[2][kMaxTerms];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int m = 0; m < kMaxTerms; ++m) {
      const int i0 = own_index(ob, p, 0), i1 = own_index(ob, p, 1);
      al[p][m] = make_float2(m < tm.n && i0 < io.n_own ? tm.own[m][i0] : 0.f,
                             m < tm.n && i1 < io.n_own ? tm.own[m][i1] : 0.f);
    }
  float2 g[2][3];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int d = 0; d < 3; ++d) g[p][d] = make_float2(0.f, 0.f);
  const int jb = sl * io.len, je = min(jb + io.len, io.n_str);
  for (int j0 = jb; j0 < je; j0 += kTile) {
    const int n = min(kTile, je - j0);
    __syncthreads();
    if ((int)threadIdx.x < n) {
      const int j = j0 + threadIdx.x;
      float4 s = io.str[j];
      if (io.str_posed) s = posed(P, s);
      sm.pt[threadIdx.x] = make_float4(s.x * sc, s.y * sc, s.z * sc, 0.f);
#pragma unroll
      for (int m = 0; m < kMaxTerms; ++m) sm.w[m][threadIdx.x] = m < tm.n ? tm.str[m][j] * wsc : 0.f;  // wsc folded in
    }
    __syncthreads();
    for (int j = 0; j < n; ++j) {
      const float4 s = sm.pt[j];
      float b[kMaxTerms];
#pragma unroll
      for (int m = 0; m < kMaxTerms; ++m) b[m] = sm.w[m][j];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const float2 dx = __fadd2_rn(dup2(s.x), q[p][0]);
        const float2 dy = __fadd2_rn(dup2(s.y), q[p][1]);
        const float2 dz = __fadd2_rn(dup2(s.z), q[p][2]);
        float2 d2 = __fmul2_rn(dx, dx);
        d2 = __ffma2_rn(dy, dy, d2);
        d2 = __ffma2_rn(dz, dz, d2);
        const float2 e = ex2_neg_pair(d2);
        float2 gs = __fmul2_rn(al[p][0], dup2(b[0]));
#pragma unroll
        for (int m = 1; m < kMaxTerms; ++m) gs = __ffma2_rn(al[p][m], dup2(b[m]), gs);
        const float2 G = __fmul2_rn(e, gs);
        g[p][0] = __ffma2_rn(G, dx, g[p][0]);
        g[p][1] = __ffma2_rn(G, dy, g[p][1]);
        g[p][2] = __ffma2_rn(G, dz, g[p][2]);
      }
    }
  }
  const float f = 2.f / T / sc;  // the differences were sc times the true ones
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const int i = own_index(ob, p, l);
      if (i < io.n_own)
#pragma unroll
        for (int d = 0; d < 3; ++d) part[((size_t)sl * 3 + d) * io.n_own + i] = f * (l ? g[p][d].y : g[p][d].x);
    }
}

// Shared memory of the combined gradient sweep's column sums.
constexpr int kG2Batch = 8;  // streamed columns per warp transpose
constexpr int kG2Stride = 36;
struct __align__(16) Grad2Smem {
  float scr[kSwT / 32][3 * kG2Batch][kG2Stride];  // per-warp transposes: (column, axis) x lane
  float wsum[kSwT / 32][3][kTile];                // per-warp column sums of a tile
};

// One tile of the combined gradient sweep (owns rows, streams the posed
// columns): the rows' partials exactly as sweep_grad_tile writes them, and
// for every streamed column j the owned block's share of dL/dz_j,
// (2/T) sum over its rows i of G_ij (x_i - z_j), into pcol[ob][d][j]. G is the
// same product the columns-owned sweep forms (same terms, same order), so one
// recomputation of K serves both sides. A column's per-lane sums (over the
// lane's 4 rows) are summed over the 32 lanes by a per-warp transpose through
// shared memory (a packed pairwise tree), then over the 4 warps in order.
__device__ __forceinline__ void sweep_grad2_tile(const SweepIO& io, const Pose12& P, float sc, float wsc, float T,
                                                 const Terms& tm, float* part, float* pcol, int ob, int sl,
                                                 SweepSmem& sm, Grad2Smem& sg) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float2 q[2][3];
  load_owned(io, P, sc, ob, q);
  float2 al[2][kMaxTerms];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int m = 0; m < kMaxTerms; ++m) {
      const int i0 = own_index(ob, p, 0), i1 = own_index(ob, p, 1);
      al[p][m] = make_float2(m < tm.n && i0 < io.n_own ? tm.own[m][i0] : 0.f,
                             m < tm.n && i1 < io.n_own ? tm.own[m][i1] : 0.f);
    }
  float2 g[2][3];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int d = 0; d < 3; ++d) g[p][d] = make_float2(0.f, 0.f);
  const float fcol = -2.f / T / sc;  // the differences were sc (z_j - x_i)
  const int jb = sl * io.len, je = min(jb + io.len, io.n_str);
  for (int j0 = jb; j0 < je; j0 += kTile) {
    const int n = min(kTile, je - j0);
    __syncthreads();  // the previous tile's points, weights and column sums are consumed
    if ((int)threadIdx.x < n) {
      const int j = j0 + threadIdx.x;
      float4 s = io.str[j];
      if (io.str_posed) s = posed(P, s);
      sm.pt[threadIdx.x] = make_float4(s.x * sc, s.y * sc, s.z * sc, 0.f);
#pragma unroll
      for (int m = 0; m < kMaxTerms; ++m) sm.w[m][threadIdx.x] = m < tm.n ? tm.str[m][j] * wsc : 0.f;  // wsc folded in
    }
    __syncthreads();
    for (int jb8 = 0; jb8 < n; jb8 += kG2Batch) {
#pragma unroll
      for (int jj = 0; jj < kG2Batch; ++jj) {
        const int j = jb8 + jj;
        float cs0 = 0.f, cs1 = 0.f, cs2 = 0.f;
        if (j < n) {  // uniform over the block
          const float4 s = sm.pt[j];
          float b[kMaxTerms];
#pragma unroll
          for (int m = 0; m < kMaxTerms; ++m) b[m] = sm.w[m][j];
          float2 c0 = make_float2(0.f, 0.f), c1 = c0, c2 = c0;
#pragma unroll
          for (int p = 0; p < 2; ++p) {
            const float2 dx = __fadd2_rn(dup2(s.x), q[p][0]);
            const float2 dy = __fadd2_rn(dup2(s.y), q[p][1]);
            const float2 dz = __fadd2_rn(dup2(s.z), q[p][2]);
            float2 d2 = __fmul2_rn(dx, dx);
            d2 = __ffma2_rn(dy, dy, d2);
            d2 = __ffma2_rn(dz, dz, d2);
            const float2 e = ex2_neg_pair(d2);
            float2 gs = __fmul2_rn(al[p][0], dup2(b[0]));
#pragma unroll
            for (int m = 1; m < kMaxTerms; ++m) gs = __ffma2_rn(al[p][m], dup2(b[m]), gs);
            const float2 G = __fmul2_rn(e, gs);
            g[p][0] = __ffma2_rn(G, dx, g[p][0]);
            g[p][1] = __ffma2_rn(G, dy, g[p][1]);
            g[p][2] = __ffma2_rn(G, dz, g[p][2]);
            c0 = __ffma2_rn(G, dx, c0);
            c1 = __ffma2_rn(G, dy, c1);
            c2 = __ffma2_rn(G, dz, c2);
          }
          cs0 = c0.x + c0.y;
          cs1 = c1.x + c1.y;
          cs2 = c2.x + c2.y;
        }
        float* col = &sg.scr[warp][3 * jj][lane];
        col[0] = cs0;
        col[kG2Stride] = cs1;
        col[2 * kG2Stride] = cs2;
      }
      __syncwarp();
      if (lane < 3 * kG2Batch) {  // value (column jj, axis d) summed over the 32 lanes
        const float4* src = reinterpret_cast<const float4*>(&sg.scr[warp][lane][0]);
        float2 t2[8];
#pragma unroll
        for (int qq = 0; qq < 8; ++qq) {
          const float4 v4 = src[qq];
          t2[qq] = __fadd2_rn(make_float2(v4.x, v4.y), make_float2(v4.z, v4.w));
        }
#pragma unroll
        for (int w = 4; w >= 1; w >>= 1)
#pragma unroll
          for (int qq = 0; qq < w; ++qq) t2[qq] = __fadd2_rn(t2[qq], t2[qq + w]);
        const int jj = lane / 3, d = lane - 3 * jj;
        sg.wsum[warp][d][jb8 + jj] = t2[0].x + t2[0].y;  // jb8 + jj < kTile
      }
      __syncwarp();
    }
    __syncthreads();
    if ((int)threadIdx.x < n) {  // the block's share of the tile's columns: the warps in order
      const int j = j0 + threadIdx.x;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float v = sg.wsum[0][d][threadIdx.x];
#pragma unroll
        for (int w = 1; w < kSwT / 32; ++w) v += sg.wsum[w][d][threadIdx.x];
        pcol[((size_t)ob * 3 + d) * io.n_str + j] = v * fcol;
      }
    }
  }
  const float f = 2.f / T / sc;  // the differences were sc times the true ones
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const int i = own_index(ob, p, l);
      if (i < io.n_own)
#pragma unroll
        for (int d = 0; d < 3; ++d) part[((size_t)sl * 3 + d) * io.n_own + i] = f * (l ? g[p][d].y : g[p][d].x);
    }
}

// The per-update launches' sweeps: one tile per block (x: owned block, y: slice).
template <int NW>
__global__ void __launch_bounds__(kSwT) k_sweep_sum(SweepIO io, const float* pose, const float* w, int ldw,
                                                    float* part) {
  __shared__ SweepSmem sm;
  float sc, wsc;
  kernel_consts(pose[kRecT], pose[kRecAlpha], sc, wsc);
  sweep_sum_tile<NW>(io, load_pose(pose), sc, wsc, w, ldw, part, blockIdx.x, blockIdx.y, sm);
}

// The combined gradient sweep (rows owned): row partials into part, the
// owned blocks' column partials into pcol.
__global__ void __launch_bounds__(kSwT, 4) k_sweep_grad2(SweepIO io, const float* pose, Terms tm, float* part,
                                                          float* pcol) {
  __shared__ SweepSmem sm;
  __shared__ Grad2Smem sg;
  const float T = pose[kRecT];
  float sc, wsc;
  kernel_consts(T, pose[kRecAlpha], sc, wsc);
  sweep_grad2_tile(io, load_pose(pose), sc, wsc, T, tm, part, pcol, blockIdx.x, blockIdx.y, sm, sg);
}


// out[m][i] (+)= sum over slices of part[sl][m][i], in slice order.
__global__ void k_reduce_slices(const float* __restrict__ part, int S, int NW, int n, float* out, int ldo, int acc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y;
  if (i >= n) return;
  float s = 0.f;
  for (int k = 0; k < S; ++k) s += part[((size_t)k * NW + m) * n + i];
  float* o = out + (size_t)m * ldo + i;
  *o = acc ? *o + s : s;
}

// ------------------------------------------------------------- O(N + M) steps
// Scalars of the backward of one update (double).
enum : int {
  kSgS = 0,     // dL/dS
  kSgXc = 9,    // dL/dXc
  kSgYc = 12,   // dL/dYc
  kSgsum = 15,  // dL/dsumM
  kScalN = 16
};

struct Vecs {
  int N, M, I1;
  const float4* X;  // X' (centred)
  const float4* Y;  // Y' (centred, unposed)
  const CenterHdr* hdr;
  const float* rec;   // the update's record (kSaTape)
  const float* s0;    // [N] input slack
  const float* u0;    // [M]
  const float* rows;  // [I1][4][N]: a^{k+1}, s^{k+1}, rs^k, r^k
  const float* cols;  // [I1][4][M]: b^{k+1}, u^{k+1}, cs^k, c^k
  const float* fin;   // [5][N]: K b, K (b (cs - 1)), K (b cs (y' - Yhat))
  float* ones;        // [M]: b^0
  float* h;           // [3][M]
  double* scal;       // kScalN
  float* g_pose;      // [12]
  float *gs, *gu;     // [N], [M]: slack adjoints (in place)
  float* ga;          // [N]
  float *gb, *gcs;    // [M]
  float* gV;          // [3][N]
  float* gp;          // [3][N]
  float* gw;          // [N]: known part of dL/dw
  float* grho;        // [N]
  float* wt4;         // [4][N]: weights of the K^T sweep (g(V), a gw)
  float* gh;          // [4][M]: K^T of wt4
  float* gr;          // [I1][N] g(r^k)
  float* gc;          // [I1][M] g(c^k)
  float* gZ;          // [3][M]
  float* gX;          // [3][N] accumulated
  float* gY;          // [3][M] accumulated
  int* cur;           // the update being differentiated (device counter, stepped down by k_pose_grad)
};

__device__ __forceinline__ const float* a_of(const Vecs& A, int k) { return A.rows + (size_t)(k - 1) * 4 * A.N; }
__device__ __forceinline__ float a_at(const Vecs& A, int k, int i) { return k == 0 ? 1.f : a_of(A, k)[i]; }
__device__ __forceinline__ float s_at(const Vecs& A, int k, int i) {
  return k == 0 ? A.s0[i] : A.rows[((size_t)(k - 1) * 4 + 1) * A.N + i];
}
__device__ __forceinline__ float rs_at(const Vecs& A, int k, int i) { return A.rows[((size_t)k * 4 + 2) * A.N + i]; }
__device__ __forceinline__ float r_at(const Vecs& A, int k, int i) { return A.rows[((size_t)k * 4 + 3) * A.N + i]; }
__device__ __forceinline__ float b_at(const Vecs& A, int k, int j) {
  return k == 0 ? 1.f : A.cols[((size_t)(k - 1) * 4) * A.M + j];
}
__device__ __forceinline__ float u_at(const Vecs& A, int k, int j) {
  return k == 0 ? A.u0[j] : A.cols[((size_t)(k - 1) * 4 + 1) * A.M + j];
}
__device__ __forceinline__ float cs_at(const Vecs& A, int k, int j) { return A.cols[((size_t)k * 4 + 2) * A.M + j]; }
__device__ __forceinline__ float c_at(const Vecs& A, int k, int j) { return A.cols[((size_t)k * 4 + 3) * A.M + j]; }
__device__ __forceinline__ double sumM_of(const Vecs& A) { return (double)A.rec[12] + (double)A.rec[13]; }

__global__ void k_fill(float* p, int n, float v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

// h_j = b_j (cs_j y_j - Yc) = b_j (cs_j y'_j - Yd + (cs_j - 1) oY), [3][M]
// (b = b^{I1}, cs = cs^{I1-1}, Yd = Yc - oY).
__device__ __forceinline__ void h_col(const Vecs& A, int j) {
  const float b = b_at(A, A.I1, j), cs = cs_at(A, A.I1 - 1, j);
  const float4 y = A.Y[j];
  const float yv[3] = {y.x, y.y, y.z};
  for (int d = 0; d < 3; ++d)
    A.h[(size_t)d * A.M + j] = b * (fmaf(cs, yv[d], -A.rec[23 + d]) + (cs - 1.f) * A.hdr->oY[d]);
}

__global__ void k_h(Vecs A) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < A.M) h_col(A, j);
}

// p_i = w_i x_i - Xc = w_i x'_i - Xc' + (w_i - 1) oX, and V_i from the final sweep's sums.
__device__ __forceinline__ void pv_of(const Vecs& A, int i, float& w, float p[3], float V[3]) {
  const float4 x = A.X[i];
  const float xv[3] = {x.x, x.y, x.z};
  const float rho = A.fin[i], m = A.fin[(size_t)A.N + i];
  w = a_of(A, A.I1)[i] * rho;
  for (int d = 0; d < 3; ++d) {
    p[d] = fmaf(w, xv[d], -A.rec[20 + d]) + (w - 1.f) * A.hdr->oX[d];
    const float yh = A.hdr->ymean[d];
    V[d] = A.fin[(size_t)(2 + d) * A.N + i] + (yh - A.rec[23 + d]) * rho + (yh + A.hdr->oY[d]) * m;
  }
}

// Horn adjoint: dL/d(R, t) of the output pose in the caller's frame (g_pose),
// where (R, t) = (R(q), Xc - R Yc) -> dL/dS, dL/dXc, dL/dYc into scal.
__device__ __forceinline__ void horn_adjoint_into(const Vecs& A, const float* g_pose, double* scal) {
  float gRo[9], gto[3], S[9], Xc[3], Yc[3], q[4], V[4][4], gS[9], gXc[3], gYc[3];
  for (int k = 0; k < 9; ++k) gRo[k] = g_pose[k];
  for (int k = 0; k < 3; ++k) gto[k] = g_pose[9 + k];
  for (int k = 0; k < 9; ++k) S[k] = A.rec[26 + k];
  for (int k = 0; k < 3; ++k) {
    Xc[k] = A.rec[14 + k];
    Yc[k] = A.rec[17 + k];
  }
  for (int k = 0; k < 4; ++k) q[k] = A.rec[35 + k];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) V[i][j] = A.rec[39 + 4 * i + j];
  horn_pose_adjoint<float>(S, Xc, Yc, q, V, gRo, gto, gS, gXc, gYc);
  for (int k = 0; k < 9; ++k) scal[kSgS + k] = gS[k];
  for (int k = 0; k < 3; ++k) {
    scal[kSgXc + k] = gXc[k];
    scal[kSgYc + k] = gYc[k];
  }
}

__global__ void k_horn_adjoint(Vecs A) { horn_adjoint_into(A, A.g_pose, A.scal); }

// Row i of S's adjoint: g(p_i) = a_i gS V_i, g(V_i) = a_i gS^T p_i, dL/da_i
// from S (S[p + 3 q] = sum a p_p V_q); adds a_i g(p_i) to v (for dL/dXc).
__device__ __forceinline__ void back_S_row(const Vecs& A, const float (&gS)[9], int i, df (&v)[3]) {
  const float* aF = a_of(A, A.I1);
  float w, p[3], Vi[3];
  pv_of(A, i, w, p, Vi);
  float ga = 0.f;
  for (int pp = 0; pp < 3; ++pp) {
    float gp = 0.f, gv = 0.f;
    for (int qq = 0; qq < 3; ++qq) {
      gp = fmaf(gS[pp + 3 * qq], Vi[qq], gp);
      gv = fmaf(gS[qq + 3 * pp], p[qq], gv);
    }
    ga = fmaf(gp, p[pp], ga);
    A.gp[(size_t)pp * A.N + i] = aF[i] * gp;
    A.gV[(size_t)pp * A.N + i] = aF[i] * gv;
    df_add(v[pp], aF[i] * gp);
  }
  A.ga[i] = ga;
}

// One block: the rows of S's adjoint; dL/dXc -= sum g(p).
__global__ void __launch_bounds__(kOneBlock) k_back_S(Vecs A) {
  __shared__ df red[3 * (kOneBlock / 32)];
  float gS[9];
  for (int k = 0; k < 9; ++k) gS[k] = (float)A.scal[kSgS + k];
  df v[3] = {df_make(0.f), df_make(0.f), df_make(0.f)};
  for (int i = threadIdx.x; i < A.N; i += blockDim.x) back_S_row(A, gS, i, v);
  block_reduce_df<3>(v, red);
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) A.scal[kSgXc + k] -= df_dbl(v[k]);
}

// Per row: the part of dL/dw known before dL/dsumM, gw = x . (g(p) + gXc/sumM);
// direct dL/dx += w (g(p) + gXc/sumM); the weights of the K^T sweep.
__device__ __forceinline__ void back_w_row(const Vecs& A, const double* scal, int i) {
  const float a = a_of(A, A.I1)[i];
  const float w = a * A.fin[i];
  const float inv = (float)(1.0 / sumM_of(A));
  const float4 x = A.X[i];
  const float xv[3] = {x.x, x.y, x.z};
  float gw = 0.f;
  for (int d = 0; d < 3; ++d) {
    const float g = fmaf((float)scal[kSgXc + d], inv, A.gp[(size_t)d * A.N + i]);
    gw = fmaf(xv[d] + A.hdr->oX[d], g, gw);
    A.gX[(size_t)d * A.N + i] += w * g;
    A.wt4[(size_t)d * A.N + i] = A.gV[(size_t)d * A.N + i];
  }
  A.gw[i] = gw;
  A.wt4[3 * (size_t)A.N + i] = a * gw;
}

__global__ void k_back_w(Vecs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.N) back_w_row(A, A.scal, i);
}

// Column j's share of dL/dYc: v += b_j g(h_j).
__device__ __forceinline__ void back_Yc_col(const Vecs& A, int j, df (&v)[3]) {
  const float b = b_at(A, A.I1, j);
  for (int d = 0; d < 3; ++d) df_add_prod(v[d], b, A.gh[(size_t)d * A.M + j]);
}

// dL/dYc -= the columns' sum; dL/dsumM = -(gXc . Xc + gYc . Yc) / sumM.
__device__ __forceinline__ void finish_Yc(const Vecs& A, const df (&v)[3], double* scal) {
  double g = 0.0;
  for (int d = 0; d < 3; ++d) {
    scal[kSgYc + d] -= df_dbl(v[d]);
    g -= scal[kSgXc + d] * (double)A.rec[14 + d] + scal[kSgYc + d] * (double)A.rec[17 + d];
  }
  scal[kSgsum] = g / sumM_of(A);
}

// One block after the K^T sweep: dL/dYc and dL/dsumM.
__global__ void __launch_bounds__(kOneBlock) k_back_Yc(Vecs A) {
  __shared__ df red[3 * (kOneBlock / 32)];
  df v[3] = {df_make(0.f), df_make(0.f), df_make(0.f)};
  for (int j = threadIdx.x; j < A.M; j += blockDim.x) back_Yc_col(A, j, v);
  block_reduce_df<3>(v, red);
  if (threadIdx.x == 0) finish_Yc(A, v, A.scal);
}

// Rows (i < N): g(rho) = a (gw + gsum); dL/da^{I1} += (gw + gsum) rho.
__device__ __forceinline__ void back_final_row(const Vecs& A, const double* scal, int i) {
  const float gsum = (float)scal[kSgsum];
  const float a = a_of(A, A.I1)[i];
  const float gw = A.gw[i] + gsum;
  A.grho[i] = a * gw;
  A.ga[i] = fmaf(gw, A.fin[i], A.ga[i]);
}

// Columns, final stage: dL/db^{I1} = (cs y - Yc) . g(h) + K^T g(rho), where
// K^T g(rho) = K^T (a gw) + gsum c^{I1-1}; dL/dcs^{I1-1} = y . (b g(h) + gYc / sumM);
// direct dL/dy += cs (b g(h) + gYc / sumM).
__device__ __forceinline__ void back_final_col(const Vecs& A, const double* scal, int j) {
  const float gsum = (float)scal[kSgsum];
  const int k = A.I1 - 1;
  const float b = b_at(A, A.I1, j), cs = cs_at(A, k, j), c = c_at(A, k, j);
  const float inv = (float)(1.0 / sumM_of(A));
  const float4 y = A.Y[j];
  const float yv[3] = {y.x, y.y, y.z};
  float gb = fmaf(gsum, c, A.gh[3 * (size_t)A.M + j]), gcs = 0.f;
  for (int d = 0; d < 3; ++d) {
    const float ghd = A.gh[(size_t)d * A.M + j];
    const float gy = fmaf(b, ghd, (float)scal[kSgYc + d] * inv);
    gb = fmaf(fmaf(cs, yv[d], -A.rec[23 + d]) + (cs - 1.f) * A.hdr->oY[d], ghd, gb);
    gcs = fmaf(yv[d] + A.hdr->oY[d], gy, gcs);
    A.gY[(size_t)d * A.M + j] += cs * gy;
  }
  A.gb[j] = gb;
  A.gcs[j] = gcs;
}

__global__ void k_back_final(Vecs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.N) {
    back_final_row(A, A.scal, i);
    return;
  }
  const int j = i - A.N;
  if (j < A.M) back_final_col(A, A.scal, j);
}

// Slice partials of a K or K^T product: the sum over slices, in order.
__device__ __forceinline__ float slices_sum(const float* part, int S, int n, int i) {
  float s = 0.f;
  for (int k = 0; k < S; ++k) s += __ldcg(part + (size_t)k * n + i);
  return s;
}

// Column pass k backward: from dL/db^{k+1} (+ the pending K^T g(r^{k+1}) slice
// partials), dL/du^{k+1} and the direct dL/dcs^k: dL/db^k, dL/du^k and
// g(c^k) = dL/dcs^k b^k. d(b/cs)/dcs = -b^{k+1}/cs: the new scalings are used
// instead of b^k/cs^2, whose square overflows FP32 at low temperature
// (K ~ e^(alpha/T)).
__device__ __forceinline__ void back_colpass(const Vecs& A, int k, const float* part, int S, int j) {
  const float bk = b_at(A, k, j), cs = cs_at(A, k, j), c = c_at(A, k, j);
  const float b1 = b_at(A, k + 1, j), u1 = u_at(A, k + 1, j);
  float gb1 = A.gb[j];
  if (part) gb1 += slices_sum(part, S, A.M, j);
  const float gu1 = A.gu[j];
  const float gcs = A.gcs[j] - fmaf(gb1, b1, gu1 * u1) / cs;
  A.gc[(size_t)k * A.M + j] = gcs * bk;
  A.gb[j] = fmaf(gcs, c, gb1 / cs);
  A.gu[j] = gu1 / cs + gcs;
  A.gcs[j] = 0.f;
}

// The same with the K^T g(r^{k+1}) sum already formed (0 for the last pass).
__device__ __forceinline__ void back_colpass_sum(const Vecs& A, int k, float pending, int j) {
  const float bk = b_at(A, k, j), cs = cs_at(A, k, j), c = c_at(A, k, j);
  const float b1 = b_at(A, k + 1, j), u1 = u_at(A, k + 1, j);
  const float gb1 = A.gb[j] + pending;
  const float gu1 = A.gu[j];
  const float gcs = A.gcs[j] - fmaf(gb1, b1, gu1 * u1) / cs;
  A.gc[(size_t)k * A.M + j] = gcs * bk;
  A.gb[j] = fmaf(gcs, c, gb1 / cs);
  A.gu[j] = gu1 / cs + gcs;
  A.gcs[j] = 0.f;
}

__global__ void k_back_colpass(Vecs A, int k, const float* part, int S) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < A.M) back_colpass(A, k, part, S, j);
}

// Row pass k backward: from dL/da^{k+1} (+ the pending K g(c^k) slice partials)
// and dL/ds^{k+1}: dL/da^k, dL/ds^k and g(r^k) = dL/drs^k a^k.
__device__ __forceinline__ void back_rowpass(const Vecs& A, int k, const float* part, int S, int i) {
  const float ak = a_at(A, k, i), rs = rs_at(A, k, i), r = r_at(A, k, i);
  const float a1 = a_at(A, k + 1, i), s1 = s_at(A, k + 1, i);
  const float ga1 = A.ga[i] + slices_sum(part, S, A.N, i);
  const float gs1 = A.gs[i];
  const float grs = -fmaf(ga1, a1, gs1 * s1) / rs;
  A.gr[(size_t)k * A.N + i] = grs * ak;
  A.ga[i] = fmaf(grs, r, ga1 / rs);
  A.gs[i] = gs1 / rs + grs;
}

// The same with the K g(c^k) sum already formed.
__device__ __forceinline__ void back_rowpass_sum(const Vecs& A, int k, float pending, int i) {
  const float ak = a_at(A, k, i), rs = rs_at(A, k, i), r = r_at(A, k, i);
  const float a1 = a_at(A, k + 1, i), s1 = s_at(A, k + 1, i);
  const float ga1 = A.ga[i] + pending;
  const float gs1 = A.gs[i];
  const float grs = -fmaf(ga1, a1, gs1 * s1) / rs;
  A.gr[(size_t)k * A.N + i] = grs * ak;
  A.ga[i] = fmaf(grs, r, ga1 / rs);
  A.gs[i] = gs1 / rs + grs;
}

__global__ void k_back_rowpass(Vecs A, int k, const float* part, int S) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < A.N) back_rowpass(A, k, part, S, i);
}

// Column j's share of the input pose's gradient (sum gz y^T, sum gz, caller
// frame y = y' + oY through oY below), and dL/dy += R^T gz.
__device__ __forceinline__ void pose_grad_col(const Vecs& A, const float (&R)[9], int j, df (&v)[12]) {
  const float4 y = A.Y[j];
  const float yv[3] = {y.x, y.y, y.z};
  const float g[3] = {A.gZ[j], A.gZ[(size_t)A.M + j], A.gZ[2 * (size_t)A.M + j]};
  for (int i = 0; i < 3; ++i) {
    for (int jj = 0; jj < 3; ++jj) df_add_prod(v[3 * i + jj], g[i], yv[jj]);
    df_add(v[9 + i], g[i]);
  }
  for (int jj = 0; jj < 3; ++jj) A.gY[(size_t)jj * A.M + j] += R[jj] * g[0] + R[3 + jj] * g[1] + R[6 + jj] * g[2];
}

// dL/d(R, t) of the input pose from the summed values.
__device__ __forceinline__ void pose_grad_from(const Vecs& A, const df (&v)[12], float* g_pose) {
  for (int i = 0; i < 3; ++i) {
    const float gt = df_val(v[9 + i]);
    g_pose[9 + i] = gt;
    for (int j = 0; j < 3; ++j) g_pose[3 * i + j] = fmaf(gt, A.hdr->oY[j], df_val(v[3 * i + j]));
  }
}

// One block: dL/dR = sum gz y^T, dL/dt = sum gz (caller frame, y = y' + oY);
// per column dL/dy += R^T gz; writes dL/d(R, t) of the input pose.
__global__ void __launch_bounds__(kOneBlock) k_pose_grad(Vecs A) {
  __shared__ df red[12 * (kOneBlock / 32)];
  float R[9];
  for (int k = 0; k < 9; ++k) R[k] = A.rec[k];
  df v[12];
  for (int k = 0; k < 12; ++k) v[k] = df_make(0.f);
  for (int j = threadIdx.x; j < A.M; j += blockDim.x) pose_grad_col(A, R, j, v);
  block_reduce_df<12>(v, red);
  if (threadIdx.x == 0) {
    pose_grad_from(A, v, A.g_pose);
    *A.cur -= 1;  // the next update back
  }
}

// The current update's tape slices into the fixed copies every other kernel of
// the update reads (so one update's launches are the same for every update).
__global__ void k_load_update(const SaUpdate* tab, const int* cur, float* rec, float* s0, float* u0, float* rows,
                              float* cols, float* fin, int N, int M, int I1, float alpha) {
  const SaUpdate U = tab[*cur];
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int i = tid; i < kSaTape; i += stride) rec[i] = i == kRecT ? U.T : i == kRecAlpha ? alpha : U.rec[i];
  for (int i = tid; i < N; i += stride) s0[i] = U.s0[i];
  for (int i = tid; i < M; i += stride) u0[i] = U.u0[i];
  const int nr = I1 * 4 * N, nc = I1 * 4 * M;
  for (int i = tid; i < nr; i += stride) rows[i] = U.rows[i];
  for (int i = tid; i < nc; i += stride) cols[i] = U.cols[i];
  for (int i = tid; i < 5 * N; i += stride) fin[i] = U.fin[i];
}

// SoA outputs and the input pose's gradient out of the accumulators.
__global__ void k_copy(float* dst, const float* src, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

// ------------------------------------------------------------- persistent backward
// Block partial records of the persistent backward: three rotating slots of
// kBwdPartNV double-float values per block (at most kBwdMaxGrid blocks).
constexpr int kBwdMaxGrid = 1200;
constexpr int kBwdPartNV = 16;

// The whole backward in one cooperative launch: the updates in reverse, each
// one the stages of the launch sequence above separated by grid barriers
// instead of launch boundaries (17 barriers per update at I1 = 3). Every block
// runs Horn's adjoint and the fixed-order reductions of the block partials
// itself, so the O(1) steps need no barrier of their own. Sweeps are split
// into (owned block, slice) tiles dealt over the blocks; the slice partials
// are summed, in slice order, by the per-point stage that consumes them.
struct BwdArgs {
  Vecs A;               // workspace vectors (tape slices set per update)
  const SaUpdate* tab;  // [nsteps] the updates' tape slices and temperatures
  long nsteps;
  float alpha;
  SweepIO rows, cols;   // rows: own X, stream Y (posed); cols: own Y (posed), stream X
  float* part_r;        // slice partials of rows-owned sweeps
  float* part_c;        // slice partials of columns-owned sweeps
  df* bpart;            // [3][gridDim.x][kBwdPartNV]
  Ctl* ctl;
  float* g_in;          // [12] dL/d(R, t) of the initial pose (written at the end)
  int* d_status;
  uint64_t timeout_ns;
};

// Sum over slices of one element's partials (part[k * stride + i], k < S),
// in slice order, with the loads issued 16 at a time ahead of the adds.
__device__ __forceinline__ float slice_sum16(const float* part, int S, size_t stride, int i) {
  float s = 0.f;
  for (int k0 = 0; k0 < S; k0 += 16) {
    float v[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = k0 + k < S ? __ldcg(part + (size_t)(k0 + k) * stride + i) : 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) s += v[k];
  }
  return s;
}

// Sum over the blocks' records of NV values into tot, in every block, in a
// fixed order: lane group g (NVP lanes, one per value) adds the records of
// blocks g, g + G, ... in order, loads issued 8 at a time, then the G group
// sums are added in order. kSwT threads.
template <int NV>
__device__ __forceinline__ void sum_block_records(const df* rec, int nblk, df* scratch, df* tot) {
  constexpr int NVP = NV <= 4 ? 4 : 16;
  constexpr int G = kSwT / NVP;
  const int v = threadIdx.x % NVP, grp = threadIdx.x / NVP;
  df a = df_make(0.f);
  if (v < NV) {
    int b = grp;
    for (; b + 7 * G < nblk; b += 8 * G) {
      float2 x[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        x[k] = __ldcg(reinterpret_cast<const float2*>(rec + (size_t)(b + k * G) * kBwdPartNV + v));
#pragma unroll
      for (int k = 0; k < 8; ++k) df_add(a, df{x[k].x, x[k].y});
    }
    for (; b < nblk; b += G) {
      const float2 x = __ldcg(reinterpret_cast<const float2*>(rec + (size_t)b * kBwdPartNV + v));
      df_add(a, df{x.x, x.y});
    }
  }
  scratch[grp * NVP + v] = a;
  __syncthreads();
  if (threadIdx.x < NV) {
    df t = scratch[threadIdx.x];
    for (int g = 1; g < G; ++g) df_add(t, scratch[g * NVP + threadIdx.x]);
    tot[threadIdx.x] = t;
  }
  __syncthreads();
}

// This block's record of NV values (summed over its threads) into slot rec.
template <int NV>
__device__ __forceinline__ void store_block_record(df (&v)[NV], df* red, df* rec) {
  block_reduce_df<NV>(v, red);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k)
      __stcg(reinterpret_cast<float2*>(rec + (size_t)blockIdx.x * kBwdPartNV + k), make_float2(v[k].hi, v[k].lo));
}

#ifndef CESA_BWD_MIN_BLOCKS
#define CESA_BWD_MIN_BLOCKS 3  // blocks per SM the register budget is set for
#endif
__global__ void __launch_bounds__(kSwT, CESA_BWD_MIN_BLOCKS) softassign_bwd_kernel(const BwdArgs B) {
  __shared__ SweepSmem sm;
  __shared__ double s_scal[kScalN];
  __shared__ float s_gpose[12];
  __shared__ df s_red[12 * (kSwT / 32)];
  __shared__ df s_scr[kSwT];
  __shared__ df s_tot[kBwdPartNV];
  const int tid = threadIdx.x, nblk = gridDim.x;
  const int gtid = blockIdx.x * kSwT + tid, gstride = nblk * kSwT;
  const int N = B.A.N, M = B.A.M, I1 = B.A.I1;
  const SweepIO& io_r = B.rows;
  const SweepIO& io_c = B.cols;
  const int nob_r = (N + kOwnBlk - 1) / kOwnBlk, nob_c = (M + kOwnBlk - 1) / kOwnBlk;
  const int units_r = nob_r * io_r.S, units_c = nob_c * io_c.S;
  unsigned epoch = 0;
  bool ok = true;
  int slot = 0;
  auto next_slot = [&]() {
    df* r = B.bpart + (size_t)slot * nblk * kBwdPartNV;
    slot = slot == 2 ? 0 : slot + 1;
    return r;
  };
  auto sync = [&](int where) {
    if (ok) ok = grid_sync(B.ctl, epoch, nblk, B.timeout_ns, where);
    return ok;
  };
  if (tid < 12) s_gpose[tid] = B.A.g_pose[tid];
  __syncthreads();

  for (long n = B.nsteps - 1; n >= 0 && ok; --n) {
    const SaUpdate U = B.tab[n];
    Vecs A = B.A;
    A.rec = U.rec;
    A.s0 = U.s0;
    A.u0 = U.u0;
    A.rows = U.rows;
    A.cols = U.cols;
    A.fin = U.fin;
    const float T = U.T;
    float sc, wsc;
    kernel_consts(T, B.alpha, sc, wsc);
    const Pose12 P = load_pose(U.rec);
    // ---- Horn's adjoint (every block), then S's adjoint per row and h per column
    if (tid == 0) horn_adjoint_into(A, s_gpose, s_scal);
    __syncthreads();
    {
      float gS[9];
      for (int k = 0; k < 9; ++k) gS[k] = (float)s_scal[kSgS + k];
      df v[3] = {df_make(0.f), df_make(0.f), df_make(0.f)};
      for (int i = gtid; i < N; i += gstride) back_S_row(A, gS, i, v);
      for (int j = gtid; j < M; j += gstride) h_col(A, j);
      store_block_record<3>(v, s_red, next_slot());
    }
    if (!sync(80)) break;
    // ---- dL/dXc, then the rows' dL/dw and the K^T sweep's weights
    {
      const df* rec = B.bpart + (size_t)((slot + 2) % 3) * nblk * kBwdPartNV;
      sum_block_records<3>(rec, nblk, s_scr, s_tot);
      if (tid == 0)
        for (int k = 0; k < 3; ++k) s_scal[kSgXc + k] -= df_dbl(s_tot[k]);
      __syncthreads();
      for (int i = gtid; i < N; i += gstride) back_w_row(A, s_scal, i);
    }
    if (!sync(81)) break;
    // ---- gh = K^T wt4 (columns own, rows stream), slice partials
    for (int u = blockIdx.x; u < units_c; u += nblk)
      sweep_sum_tile<4>(io_c, P, sc, wsc, A.wt4, N, B.part_c, u % nob_c, u / nob_c, sm);
    if (!sync(82)) break;
    // ---- gh summed per (column, weight); the columns' share of dL/dYc
    {
      df v[3] = {df_make(0.f), df_make(0.f), df_make(0.f)};
      for (int it = gtid; it < 4 * M; it += gstride) {
        const int m = it / M, j = it - m * M;
        const float g = slice_sum16(B.part_c + (size_t)m * M, io_c.S, (size_t)4 * M, j);
        A.gh[(size_t)m * M + j] = g;
        if (m < 3) df_add_prod(v[m], b_at(A, I1, j), g);
      }
      store_block_record<3>(v, s_red, next_slot());
    }
    if (!sync(83)) break;
    // ---- dL/dYc, dL/dsumM; the final stage per row and column, fused with the
    //      backward of the last column pass (column-local)
    {
      const df* rec = B.bpart + (size_t)((slot + 2) % 3) * nblk * kBwdPartNV;
      sum_block_records<3>(rec, nblk, s_scr, s_tot);
      if (tid == 0) {
        df v[3] = {s_tot[0], s_tot[1], s_tot[2]};
        finish_Yc(A, v, s_scal);
      }
      __syncthreads();
      for (int i = gtid; i < N; i += gstride) back_final_row(A, s_scal, i);
      for (int j = gtid; j < M; j += gstride) {
        back_final_col(A, s_scal, j);
        back_colpass_sum(A, I1 - 1, 0.f, j);
      }
    }
    if (!sync(84)) break;
    // ---- the row and column passes in reverse
    for (int k = I1 - 1; k >= 0; --k) {
      // dL/da^{k+1} += K g(c^k): rows own, columns stream
      for (int u = blockIdx.x; u < units_r; u += nblk)
        sweep_sum_tile<1>(io_r, P, sc, wsc, A.gc + (size_t)k * M, M, B.part_r, u % nob_r, u / nob_r, sm);
      if (!sync(85)) break;
      for (int i = gtid; i < N; i += gstride) back_rowpass_sum(A, k, slice_sum16(B.part_r, io_r.S, N, i), i);
      if (!sync(86)) break;
      if (k == 0) break;
      // dL/db^k += K^T g(r^k), then the column pass k - 1 (b^0 = 1 is a constant)
      for (int u = blockIdx.x; u < units_c; u += nblk)
        sweep_sum_tile<1>(io_c, P, sc, wsc, A.gr + (size_t)k * N, N, B.part_c, u % nob_c, u / nob_c, sm);
      if (!sync(87)) break;
      for (int j = gtid; j < M; j += gstride) back_colpass_sum(A, k - 1, slice_sum16(B.part_c, io_c.S, M, j), j);
      if (!sync(88)) break;
    }
    if (!ok) break;
    // ---- the gradient sweeps: dL/dx (rows own) and dL/dz (columns own), in
    //      chunks of kMaxTerms rank-1 terms of dL/dK
    const int nterms = 4 + 2 * I1;
    for (int t0 = 0; t0 < nterms && ok; t0 += kMaxTerms) {
      Terms tr{}, tc{};
      tr.n = tc.n = min(kMaxTerms, nterms - t0);
      for (int m = 0; m < tr.n; ++m) {
        const int t = t0 + m;
        const float *ta, *tb;
        if (t < 3) {
          ta = A.gV + (size_t)t * N;
          tb = A.h + (size_t)t * M;
        } else if (t == 3) {
          ta = A.grho;
          tb = A.cols + (size_t)(I1 - 1) * 4 * M;  // b^{I1}
        } else if (t < 4 + I1) {
          const int k = t - 4;
          ta = A.rows + (size_t)k * 4 * N;  // a^{k+1}
          tb = A.gc + (size_t)k * M;
        } else {
          const int k = t - 4 - I1;
          ta = A.gr + (size_t)k * N;
          tb = k == 0 ? A.ones : A.cols + (size_t)(k - 1) * 4 * M;  // b^k
        }
        tr.own[m] = ta;
        tr.str[m] = tb;
        tc.own[m] = tb;
        tc.str[m] = ta;
      }
      for (int u = blockIdx.x; u < units_r + units_c; u += nblk) {
        if (u < units_r)
          sweep_grad_tile(io_r, P, sc, wsc, T, tr, B.part_r, u % nob_r, u / nob_r, sm);
        else
          sweep_grad_tile(io_c, P, sc, wsc, T, tc, B.part_c, (u - units_r) % nob_c, (u - units_r) / nob_c, sm);
      }
      if (!sync(89)) break;
      const bool last = t0 + kMaxTerms >= nterms;
      float R[9];
      for (int k = 0; k < 9; ++k) R[k] = U.rec[k];
      df v[12];
      for (int k = 0; k < 12; ++k) v[k] = df_make(0.f);
      for (int it = gtid; it < 3 * N; it += gstride) {
        const int d = it / N, i = it - d * N;
        A.gX[(size_t)d * N + i] += slice_sum16(B.part_r + (size_t)d * N, io_r.S, (size_t)3 * N, i);
      }
      for (int it = gtid; it < 3 * M; it += gstride) {
        const int d = it / M, j = it - d * M;
        float g = slice_sum16(B.part_c + (size_t)d * M, io_c.S, (size_t)3 * M, j);
        if (t0 > 0) g += A.gZ[(size_t)d * M + j];
        A.gZ[(size_t)d * M + j] = g;
        if (last) {  // this component's share of sum gz y^T and sum gz
          const float4 y = A.Y[j];
          df_add_prod(v[3 * d], g, y.x);
          df_add_prod(v[3 * d + 1], g, y.y);
          df_add_prod(v[3 * d + 2], g, y.z);
          df_add(v[9 + d], g);
        }
      }
      if (last) store_block_record<12>(v, s_red, next_slot());
      if (!sync(90)) break;
      if (last) {
        // dL/dy += R^T gz (all three components of gz are in place now)
        for (int j = gtid; j < M; j += gstride) {
          const float g[3] = {A.gZ[j], A.gZ[(size_t)M + j], A.gZ[2 * (size_t)M + j]};
          for (int jj = 0; jj < 3; ++jj) A.gY[(size_t)jj * M + j] += R[jj] * g[0] + R[3 + jj] * g[1] + R[6 + jj] * g[2];
        }
        // dL/d(R, t) of this update's input pose = the output pose of the update before
        const df* rec = B.bpart + (size_t)((slot + 2) % 3) * nblk * kBwdPartNV;
        sum_block_records<12>(rec, nblk, s_scr, s_tot);
        if (tid == 0) {
          df t[12];
          for (int k = 0; k < 12; ++k) t[k] = s_tot[k];
          pose_grad_from(A, t, s_gpose);
        }
        __syncthreads();
      }
    }
  }
  if (blockIdx.x == 0 && tid == 0) {
    const int st = ld_status(B.ctl);
    if (st == kStatusOk)
      for (int k = 0; k < 12; ++k) B.g_in[k] = s_gpose[k];
    if (B.d_status) *B.d_status = st;
  }
}

// ------------------------------------------------------------------ host side
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

struct Plan {
  SweepIO rows, cols;  // own X / stream Y; own Y / stream X
};

// Slices so that a sweep has about 1200 blocks (8 per SM of 152), each slice
// at least 32 streamed points (small clouds get short slices rather than an
// under-filled grid).
void plan_side(SweepIO& io, int n_own, int n_str) {
  const int nb = (n_own + kOwnBlk - 1) / kOwnBlk;
  const int max_s = std::max(1, (n_str + 31) / 32);
  io.S = std::max(1, std::min(max_s, (1200 + nb - 1) / nb));
  io.len = (n_str + io.S - 1) / io.S;
  io.S = (n_str + io.len - 1) / io.len;
  io.n_own = n_own;
  io.n_str = n_str;
}

Plan make_plan(int N, int M) {
  Plan P{};
  plan_side(P.rows, N, M);
  plan_side(P.cols, M, N);
  P.rows.own_posed = false;
  P.rows.str_posed = true;
  P.cols.own_posed = true;
  P.cols.str_posed = false;
  return P;
}

struct Layout {
  Vecs V;
  Ctl* ctl;      // status and grid-barrier counter of the persistent backward
  float* part;   // slice partials (rows-owned sweeps in the persistent backward)
  float* part2;  // slice partials of the columns-owned sweeps (persistent backward)
  df* bpart;     // [3][kBwdMaxGrid][kBwdPartNV]
  float *rec, *s0, *u0, *rows, *cols, *fin;  // the current update's tape slices (copies)
  float4 *X, *Y;                             // the packed clouds (copies)
  CenterHdr* hdr;
  SaUpdate* tab;                             // [nsteps]
  size_t total;
};

Layout carve(void* base, int N, int M, int I1, long nsteps, const Plan& P) {
  Carve c(base);
  Layout L{};
  Vecs& A = L.V;
  A.N = N;
  A.M = M;
  A.I1 = I1;
  L.ctl = c.take<Ctl>(1);  // first: read_ws_status reads the status here
  A.cur = c.take<int>(1);
  A.g_pose = c.take<float>(16);
  A.gs = c.take<float>(N);
  A.gu = c.take<float>(M);
  A.gX = c.take<float>(3 * (size_t)N);
  A.gY = c.take<float>(3 * (size_t)M);
  A.ones = c.take<float>(M);
  A.h = c.take<float>(3 * (size_t)M);
  A.scal = c.take<double>(kScalN);
  A.ga = c.take<float>(N);
  A.gb = c.take<float>(M);
  A.gcs = c.take<float>(M);
  A.gV = c.take<float>(3 * (size_t)N);
  A.gp = c.take<float>(3 * (size_t)N);
  A.gw = c.take<float>(N);
  A.grho = c.take<float>(N);
  A.wt4 = c.take<float>(4 * (size_t)N);
  A.gh = c.take<float>(4 * (size_t)M);
  A.gr = c.take<float>((size_t)I1 * N);
  A.gc = c.take<float>((size_t)I1 * M);
  A.gZ = c.take<float>(3 * (size_t)M);
  L.rec = c.take<float>(kSaTape);
  L.s0 = c.take<float>(N);
  L.u0 = c.take<float>(M);
  L.rows = c.take<float>((size_t)I1 * 4 * N);
  L.cols = c.take<float>((size_t)I1 * 4 * M);
  L.fin = c.take<float>(5 * (size_t)N);
  L.X = c.take<float4>(N);
  L.Y = c.take<float4>(M);
  L.hdr = c.take<CenterHdr>(1);
  A.rec = L.rec;
  A.s0 = L.s0;
  A.u0 = L.u0;
  A.rows = L.rows;
  A.cols = L.cols;
  A.fin = L.fin;
  const size_t pr = (size_t)P.rows.S * 4 * N, pc = (size_t)P.cols.S * 4 * M;
  const size_t pcol = (size_t)((N + kOwnBlk - 1) / kOwnBlk) * 3 * M;  // the combined gradient sweep's column partials
  L.part = c.take<float>(std::max(pr, pc));
  L.part2 = c.take<float>(std::max(std::max(pr, pc), pcol));
  L.bpart = c.take<df>((size_t)3 * kBwdMaxGrid * kBwdPartNV);
  // last, so that every other offset is the same whatever the schedule's length
  L.tab = c.take<SaUpdate>((size_t)(nsteps > 0 ? nsteps : 1));
  L.total = c.off;
  return L;
}

int blocks(int n) { return (n + kGlue - 1) / kGlue; }

// Slice partials of NW K-products of weight vectors into part (rows: K w, w
// over columns; columns: K^T w, w over rows).
template <int NW>
void sweep_partials(const SweepIO& io, float* part, const float* rec, const float* w, int ldw, cudaStream_t st) {
  dim3 g((io.n_own + kOwnBlk - 1) / kOwnBlk, io.S);
  k_sweep_sum<NW><<<g, kSwT, 0, st>>>(io, rec, w, ldw, part);
}

// out[m] (+)= the slice-ordered sums of a sweep's partials.
template <int NW>
void sum_sweep(const SweepIO& io, const Layout& L, const float* w, int ldw, float* out, int ldo, bool acc,
               cudaStream_t st) {
  sweep_partials<NW>(io, L.part, L.rec, w, ldw, st);
  k_reduce_slices<<<dim3(blocks(io.n_own), NW), kGlue, 0, st>>>(L.part, io.S, NW, io.n_own, out, ldo, acc ? 1 : 0);
}

// dL/dx (added to gx) and dL/dz (gz; added when acc) of a chunk of terms by
// one rows-owned sweep: its slice partials, then the owned blocks' column
// partials, each summed in order.
void grad2_sweep(const SweepIO& io, const Layout& L, const Terms& tm, float* gx, float* gz, bool acc, cudaStream_t st) {
  const int nob = (io.n_own + kOwnBlk - 1) / kOwnBlk;
  k_sweep_grad2<<<dim3(nob, io.S), kSwT, 0, st>>>(io, L.rec, tm, L.part, L.part2);
  k_reduce_slices<<<dim3(blocks(io.n_own), 3), kGlue, 0, st>>>(L.part, io.S, 3, io.n_own, gx, io.n_own, 1);
  k_reduce_slices<<<dim3(blocks(io.n_str), 3), kGlue, 0, st>>>(L.part2, nob, 3, io.n_str, gz, io.n_str, acc ? 1 : 0);
}

struct Ctx {
  Plan P;
  Layout L;
  Vecs A;
};

int make_ctx(const SoftassignBackward& B, void* ws, size_t ws_bytes, Ctx& c) {
  const int N = B.N, M = B.M, I1 = B.I1;
  if (N < 1 || M < 1 || I1 < 1 || 4 + 2 * I1 > 64 || B.nsteps < 0) return (int)cudaErrorInvalidValue;
  c.P = make_plan(N, M);
  c.L = carve(ws, N, M, I1, B.nsteps, c.P);
  if (!ws || c.L.total > ws_bytes) return (int)cudaErrorInvalidValue;
  // every launch reads the workspace copies of the clouds, so that one
  // update's launches do not depend on where the tape lives
  c.P.rows.own = c.L.X;
  c.P.rows.str = c.L.Y;
  c.P.cols.own = c.L.Y;
  c.P.cols.str = c.L.X;
  c.A = c.L.V;
  c.A.X = c.L.X;
  c.A.Y = c.L.Y;
  c.A.hdr = c.L.hdr;
  return 0;
}

}  // namespace

size_t softassign_bwd_ws_need(int N, int M, int I1, long nsteps) {
  const Plan P = make_plan(N, M);
  return carve(nullptr, N, M, I1, nsteps, P).total;
}

int softassign_bwd_prepare(const SoftassignBackward& B, const SaUpdate* host_tab, void* ws, size_t ws_bytes,
                           cudaStream_t st) {
  Ctx c;
  int r = make_ctx(B, ws, ws_bytes, c);
  if (r) return r;
  const int N = B.N, M = B.M;
  const int last = (int)B.nsteps - 1;
  cudaError_t e = cudaSuccess;
  if (B.nsteps > 0)
    e = cudaMemcpyAsync(c.L.tab, host_tab, sizeof(SaUpdate) * (size_t)B.nsteps, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.A.cur, &last, sizeof(int), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.L.X, B.X, sizeof(float4) * (size_t)N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.L.Y, B.Y, sizeof(float4) * (size_t)M, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.L.hdr, B.hdr, sizeof(CenterHdr), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.A.g_pose, B.g_out, sizeof(float) * 12, cudaMemcpyDeviceToDevice, st);
  // the output slack of the last update does not feed the loss
  if (e == cudaSuccess) e = cudaMemsetAsync(c.A.gs, 0, sizeof(float) * N, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(c.A.gu, 0, sizeof(float) * M, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(c.A.gX, 0, sizeof(float) * 3 * (size_t)N, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(c.A.gY, 0, sizeof(float) * 3 * (size_t)M, st);
  if (e != cudaSuccess) return (int)e;
  k_fill<<<std::min(blocks(M), 1024), kGlue, 0, st>>>(c.A.ones, M, 1.f);
  return (int)cudaGetLastError();
}

// The launches of one update's backward, the update chosen on the device (the
// same launches, with the same arguments, for every update).
int softassign_bwd_update(const SoftassignBackward& B, void* ws, size_t ws_bytes, cudaStream_t st) {
  Ctx c;
  int r = make_ctx(B, ws, ws_bytes, c);
  if (r) return r;
  const Plan& P = c.P;
  const Layout& L = c.L;
  Vecs& A = c.A;
  const int N = B.N, M = B.M, I1 = B.I1;
  const int ob = one_block_threads(std::max(N, M));
  {
    const int total = 4 * I1 * (N + M) + 6 * N + M;
    const int g = std::min(std::max(1, (total + 4 * kGlue - 1) / (4 * kGlue)), 1024);
    k_load_update<<<g, kGlue, 0, st>>>(L.tab, A.cur, L.rec, L.s0, L.u0, L.rows, L.cols, L.fin, N, M, I1, B.alpha);
  }
  // ---- final stage and Horn
  k_h<<<blocks(M), kGlue, 0, st>>>(A);
  k_horn_adjoint<<<1, 1, 0, st>>>(A);
  k_back_S<<<1, ob, 0, st>>>(A);
  k_back_w<<<blocks(N), kGlue, 0, st>>>(A);
  sum_sweep<4>(P.cols, L, A.wt4, N, A.gh, M, false, st);
  k_back_Yc<<<1, ob, 0, st>>>(A);
  k_back_final<<<blocks(N + M), kGlue, 0, st>>>(A);
  // ---- the column and row passes in reverse; each K / K^T product's slice
  // partials are summed by the kernel that consumes them
  const float* pending = nullptr;
  for (int k = I1 - 1; k >= 0; --k) {
    k_back_colpass<<<blocks(M), kGlue, 0, st>>>(A, k, pending, P.cols.S);
    // dL/da^{k+1} += K g(c^k)
    sweep_partials<1>(P.rows, L.part, L.rec, A.gc + (size_t)k * M, M, st);
    k_back_rowpass<<<blocks(N), kGlue, 0, st>>>(A, k, L.part, P.rows.S);
    // dL/db^k += K^T g(r^k); b^0 = 1 is a constant
    pending = nullptr;
    if (k >= 1) {
      sweep_partials<1>(P.cols, L.part, L.rec, A.gr + (size_t)k * N, N, st);
      pending = L.part;
    }
  }
  // ---- rank-1 terms of dL/dK (rows: alpha, columns: beta)
  const int nterms = 4 + 2 * I1;
  const float* ta[64];
  const float* tb[64];
  for (int d = 0; d < 3; ++d) {
    ta[d] = A.gV + (size_t)d * N;
    tb[d] = A.h + (size_t)d * M;
  }
  ta[3] = A.grho;
  tb[3] = L.cols + (size_t)(I1 - 1) * 4 * M;  // b^{I1}
  for (int k = 0; k < I1; ++k) {
    ta[4 + k] = L.rows + (size_t)k * 4 * N;  // a^{k+1}
    tb[4 + k] = A.gc + (size_t)k * M;
    ta[4 + I1 + k] = A.gr + (size_t)k * N;
    tb[4 + I1 + k] = k == 0 ? A.ones : L.cols + (size_t)(k - 1) * 4 * M;  // b^k
  }
  for (int t0 = 0; t0 < nterms; t0 += kMaxTerms) {
    Terms tr{};
    tr.n = std::min(kMaxTerms, nterms - t0);
    for (int m = 0; m < tr.n; ++m) {
      tr.own[m] = ta[t0 + m];
      tr.str[m] = tb[t0 + m];
    }
    grad2_sweep(P.rows, L, tr, A.gX, A.gZ, t0 > 0, st);
  }
  k_pose_grad<<<1, ob, 0, st>>>(A);
  return (int)cudaGetLastError();
}

int softassign_bwd_finish(const SoftassignBackward& B, void* ws, size_t ws_bytes, cudaStream_t st) {
  Ctx c;
  int r = make_ctx(B, ws, ws_bytes, c);
  if (r) return r;
  const int N = B.N, M = B.M;
  k_copy<<<std::min(blocks(3 * N), 1024), kGlue, 0, st>>>(B.gX, c.A.gX, 3 * N);
  k_copy<<<std::min(blocks(3 * M), 1024), kGlue, 0, st>>>(B.gY, c.A.gY, 3 * M);
  k_copy<<<1, 32, 0, st>>>(B.g_in, c.A.g_pose, 12);
  return (int)cudaGetLastError();
}

namespace {
// Slices of a sweep in the persistent backward: enough tiles to about fill the
// grid, slices of at least 64 streamed points, and no more slices than the
// workspace's partial buffers hold (the launch sequence's plan, S_cap).
void plan_persistent(SweepIO& io, int grid, int S_cap) {
  const int nb = (io.n_own + kOwnBlk - 1) / kOwnBlk;
  int S = std::max(1, grid / nb);
  S = std::min(S, std::max(1, (io.n_str + 63) / 64));
  S = std::min(S, std::max(1, S_cap));
  io.len = (io.n_str + S - 1) / S;
  io.S = (io.n_str + io.len - 1) / io.len;
}
}  // namespace

int softassign_bwd_persistent(const SoftassignBackward& B, const SaUpdate* host_tab, void* ws, size_t ws_bytes,
                              cudaStream_t st, int* d_status, uint64_t timeout_ns) {
  Ctx c;
  int r = make_ctx(B, ws, ws_bytes, c);
  if (r) return r;
  int device = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, softassign_bwd_kernel, kSwT, 0);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorCooperativeLaunchTooLarge;
  // Blocks: one per SM at least, more (up to the resident limit) while there
  // are 32 points of X and Y per block. Every block reduces all blocks'
  // records three times per update, so small problems run on fewer blocks.
  const int N = B.N, M = B.M;
  const int want = std::max(sms, (int)(((long)N + M) / 32));
  const int grid = std::min(std::min(per_sm * sms, kBwdMaxGrid), want);
  const Layout& L = c.L;
  e = cudaMemsetAsync(L.ctl, 0, sizeof(Ctl), st);
  if (e == cudaSuccess && B.nsteps > 0)
    e = cudaMemcpyAsync(L.tab, host_tab, sizeof(SaUpdate) * (size_t)B.nsteps, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(L.X, B.X, sizeof(float4) * (size_t)N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(L.Y, B.Y, sizeof(float4) * (size_t)M, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(L.hdr, B.hdr, sizeof(CenterHdr), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.A.g_pose, B.g_out, sizeof(float) * 12, cudaMemcpyDeviceToDevice, st);
  // the output slack of the last update does not feed the loss; dL/dX, dL/dY accumulate in the outputs
  if (e == cudaSuccess) e = cudaMemsetAsync(c.A.gs, 0, sizeof(float) * N, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(c.A.gu, 0, sizeof(float) * M, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B.gX, 0, sizeof(float) * 3 * (size_t)N, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B.gY, 0, sizeof(float) * 3 * (size_t)M, st);
  if (e != cudaSuccess) return (int)e;
  k_fill<<<std::min(blocks(M), 1024), kGlue, 0, st>>>(c.A.ones, M, 1.f);
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  BwdArgs a{};
  a.A = c.A;
  a.A.gX = B.gX;
  a.A.gY = B.gY;
  a.tab = L.tab;
  a.nsteps = B.nsteps;
  a.alpha = B.alpha;
  a.rows = c.P.rows;
  a.cols = c.P.cols;
  plan_persistent(a.rows, grid, c.P.rows.S);
  plan_persistent(a.cols, grid, c.P.cols.S);
  a.part_r = L.part;
  a.part_c = L.part2;
  a.bpart = L.bpart;
  a.ctl = L.ctl;
  a.g_in = B.g_in;
  a.d_status = d_status;
  a.timeout_ns = timeout_ns;
  void* args[] = {(void*)&a};
  return (int)cudaLaunchCooperativeKernel((const void*)softassign_bwd_kernel, dim3(grid), dim3(kSwT), args, 0, st);
}

}  // namespace cesa
