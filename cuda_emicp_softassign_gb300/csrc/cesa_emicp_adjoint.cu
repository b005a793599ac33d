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
//      (z_r = R y_r + t) for (row block, column slice) units and forms, per
//      element, ge = gA_r + gB_r . x_c + 2 e gC_r (the adjoints of the row sums
//      A = sum e, B = sum e x, C = sum e^2 + outlier) and w = e ge / s2:
//        dL/dz_r += w (x_c - z_r)            (per row, in registers)
//        dL/dx_c += e gB_r - w (x_c - z_r)   (per column, reduced over the
//                                             block's 128 rows by a warp
//                                             reduce-scatter, one partial per
//                                             row block and column);
//   3. the block that completes a row block (split completion over slices)
//      adds dL/dy_r = R^T dL/dz_r + lambda_r gP + gQ^T u_r and writes the row
//      block's record of sum dL/dz_r y_r^T (row-major, as R), sum dL/dz_r and, for rows on the
//      C_r <= 1e-6 branch (lambda = 1, u = mean X), sum gu_r;
//   4. after the grid barrier every block reduces the records (the upstream
//      gradient of the previous step's pose) and adds, for its share of the
//      columns, the row-block partials of dL/dx_c in a fixed order.
// Per element: 6 (distance) + 1 (exponent) + 4 (ge) + 1 (w, with 1/s2 folded
// into the row coefficients) + 3 (dz) + 6 (dx) FP32 ops + 1 MUFU, against
// 12 + 1 in the forward, on packed pairs of rows (FFMA2/FADD2/FMUL2).
#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {
namespace {

constexpr int kColGroup = 4;  // columns per warp reduce-scatter (4 columns x 4 components)
constexpr int kPairs2 = 2 * kPairs;  // packed row pairs per lane: 4 rows of each of two row blocks

struct EmAdjArgs {
  const float4* rows;  // Y' centred (M)
  const float4* cols;  // X' centred (N)
  int M, N;
  SweepGeom geo;  // own rows (M), stream columns (N)
  int nsteps;
  const float* tape;      // [nsteps][kEmTape]
  const float* row_tape;  // [nsteps][M][5]
  const float* g_out;     // dL/d(R, t) of the final pose (device, caller frame)
  const CenterHdr* hdr;   // centring offsets (t' = t + R oY - oX)
  float4* gX;             // [N] accumulated (centred = caller frame)
  float4* gY;             // [M]
  float* g_in;            // [12] dL/d(R, t) of the initial pose, caller frame
  float* part;            // split partials [units][3][128]
  unsigned* cnt;          // [nblk]
  df* rec;                // [2][nblk][16]
  float4* part_x;         // [2][ceil(nblk / 2)][N]: one partial per pair of row blocks
  Ctl* ctl;
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

// Sum over the 32 lanes of v[k] for k = 0..15; lane l receives the sum for
// k = l & 15 (a fold of the two half-warps, then a reduce-scatter).
__device__ __forceinline__ float reduce_scatter16(float (&v)[16]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], 16);
#pragma unroll
  for (int m = 8, n = 8; m >= 1; m >>= 1, n >>= 1) {
    const bool up = lane & m;
#pragma unroll
    for (int i = 0; i < n; ++i) {
      const float send = up ? v[i] : v[i + n];
      const float keep = up ? v[i + n] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, m);
    }
  }
  return v[0];
}

// Per owned row: z (posed), and the row-sum adjoints gA, gB[3], gC (zero for
// rows on the C <= 1e-6 branch and for rows past M).
struct RowCoef {
  float z[3];
  float gA, gB[3], gC2;  // gC2 = 2 gC
};

__device__ __forceinline__ RowCoef row_coef(const float4 y, bool valid, const float* rt, const float (&R)[9],
                                            const float (&t)[3], const float (&coef)[16]) {
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
  float4 raw[2][kChunk];
  float4 prep[kChunk];
  float red[kMaxAcc][kWarps][kBlockPts];
  uint64_t full[2];
  int flag;
};

__global__ void __launch_bounds__(kThreads, 1) emicp_adjoint_kernel(const EmAdjArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  AdjSmem& sm = *reinterpret_cast<AdjSmem*>(smem_raw);
  __shared__ float s_g[12];     // dL/d(R, t') of the current step's output pose
  __shared__ float s_coef[16];  // moment adjoints of the current step
  __shared__ float s_pose[13];  // the step's input pose and sigma_p2
  __shared__ df s_red[kThreads];
  __shared__ df s_tot[16];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned G = gridDim.x;
  const SweepGeom& g = A.geo;
  if (tid == 0) {
    for (int s = 0; s < 2; ++s) mbar_init(&sm.full[s], 1);
    mbar_init_fence();
    // caller frame -> centred frame: t = t' + oX - R oY, so dL/dt' = dL/dt and
    // dL/dR' = dL/dR - dL/dt oY^T
    for (int i = 0; i < 3; ++i) {
      s_g[9 + i] = A.g_out[9 + i];
      for (int j = 0; j < 3; ++j) s_g[3 * i + j] = A.g_out[3 * i + j] - A.g_out[9 + i] * A.hdr->oY[j];
    }
  }
  __syncthreads();
  unsigned uses[2] = {0u, 0u};
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
    float R[9], t[3], coef[16];
    for (int i = 0; i < 9; ++i) R[i] = s_pose[i];
    for (int i = 0; i < 3; ++i) t[i] = s_pose[9 + i];
    for (int i = 0; i < 16; ++i) coef[i] = s_coef[i];
    const float s2 = s_pose[12];
    const float nk = -kLog2e / (2.f * s2), inv_s2 = 1.f / s2;
    const float* rtape = A.row_tape + (size_t)k * A.M * 5;
    df* recs = A.rec + (size_t)par * g.nblk * 16;
    float4* px = A.part_x + (size_t)par * ((g.nblk + 1) / 2) * A.N;

    // units: (pair of row blocks, slice); a lane holds 4 rows of each row block
    const int nb2 = (g.nblk + 1) / 2;
    for (int u = blockIdx.x; u < g.units && ok; u += G) {
      const int b2 = u / g.slices, sl = u - b2 * g.slices;
      const int cb = sl * g.slice_len, ce = min(cb + g.slice_len, g.n_stream);
      // rows in packed pairs: pair P = 2 h + k holds rows (2k, 2k + 1) of row
      // block 2 b2 + h: -z, gA, gB, 2 gC (all scaled by 1/s2), and dL/dz
      float2 nz[kPairs2][3], pgA[kPairs2], pgB[kPairs2][3], pgC[kPairs2], gz2[kPairs2][3];
#pragma unroll
      for (int P = 0; P < kPairs2; ++P) {
        RowCoef c2[2];
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          const int r = (2 * b2 + (P >> 1)) * kBlockPts + lane + 32 * (2 * (P & 1) + hh);
          const bool valid = r < A.M;
          const float4 y = valid ? ld_cg(A.rows + r) : make_float4(0.f, 0.f, 0.f, 0.f);
          c2[hh] = row_coef(y, valid, rtape + (size_t)(valid ? r : 0) * 5, R, t, coef);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          nz[P][a] = make_float2(-c2[0].z[a], -c2[1].z[a]);
          pgB[P][a] = make_float2(c2[0].gB[a] * inv_s2, c2[1].gB[a] * inv_s2);
          gz2[P][a] = make_float2(0.f, 0.f);
        }
        pgA[P] = make_float2(c2[0].gA * inv_s2, c2[1].gA * inv_s2);
        pgC[P] = make_float2(c2[0].gC2 * inv_s2, c2[1].gC2 * inv_s2);
      }
      int st = 0;
      uses[0] += 1;
      if (tid == 0) {
        const int len = min(kChunk, ce - cb);
        mbar_arrive_expect_tx(&sm.full[0], (unsigned)len * 16u);
        bulk_g2s(&sm.raw[0][0], A.cols + cb, (unsigned)len * 16u, &sm.full[0]);
      }
      for (int first = cb; first < ce; first += kChunk) {
        const int len = min(kChunk, ce - first);
        const int nst = st ^ 1;
        const bool more = first + kChunk < ce;
        if (more) {
          uses[nst] += 1;
          if (tid == 0) {
            const int nlen = min(kChunk, ce - first - kChunk);
            mbar_arrive_expect_tx(&sm.full[nst], (unsigned)nlen * 16u);
            bulk_g2s(&sm.raw[nst][0], A.cols + first + kChunk, (unsigned)nlen * 16u, &sm.full[nst]);
          }
        }
        const bool bad = !mbar_wait(&sm.full[st], (uses[st] - 1u) & 1u, A.ctl, A.timeout_ns, 100);
        if (__syncthreads_or(bad)) {
          if (more) mbar_wait(&sm.full[nst], (uses[nst] - 1u) & 1u, A.ctl, A.timeout_ns, 101);
          ok = false;
          break;
        }
        // columns past the chunk's end in the last group: points so far away that
        // their affinity is exactly 0, so every term they feed is 0
        if (tid < kColGroup - 1 && len + tid < kChunk)
          sm.raw[st][len + tid] = make_float4(1e18f, 1e18f, 1e18f, 0.f);
        __syncthreads();
        const float4* xs = sm.raw[st];
        // groups of 4 columns per warp: per column, 8 rows per lane, then the
        // 4 x 4 column partials (x, y, z, pad) reduce-scattered over the lanes
        for (int c0 = warp * kColGroup; c0 < len; c0 += kWarps * kColGroup) {
          float v[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) v[i] = 0.f;
#pragma unroll
          for (int cc = 0; cc < kColGroup; ++cc) {
            {
              const float4 x = xs[c0 + cc];
              const float2 xx = dup2(x.x), xy = dup2(x.y), xz = dup2(x.z);
              float2 vx = make_float2(0.f, 0.f), vy = vx, vz = vx;  // sum e gB'
              float2 ux = vx, uy = vx, uz = vx;                       // sum w (x - z)
#pragma unroll
              for (int P = 0; P < kPairs2; ++P) {
                const float2 dx = __fadd2_rn(xx, nz[P][0]);
                const float2 dy = __fadd2_rn(xy, nz[P][1]);
                const float2 dz = __fadd2_rn(xz, nz[P][2]);
                float2 d2 = __fmul2_rn(dx, dx);
                d2 = __ffma2_rn(dy, dy, d2);
                d2 = __ffma2_rn(dz, dz, d2);
                const float2 e = ex2_pair(__fmul2_rn(d2, dup2(nk)));
                float2 ge = __ffma2_rn(pgB[P][0], xx, pgA[P]);
                ge = __ffma2_rn(pgB[P][1], xy, ge);
                ge = __ffma2_rn(pgB[P][2], xz, ge);
                ge = __ffma2_rn(e, pgC[P], ge);
                const float2 w = __fmul2_rn(e, ge);
                gz2[P][0] = __ffma2_rn(w, dx, gz2[P][0]);
                gz2[P][1] = __ffma2_rn(w, dy, gz2[P][1]);
                gz2[P][2] = __ffma2_rn(w, dz, gz2[P][2]);
                ux = __ffma2_rn(w, dx, ux);
                uy = __ffma2_rn(w, dy, uy);
                uz = __ffma2_rn(w, dz, uz);
                vx = __ffma2_rn(e, pgB[P][0], vx);
                vy = __ffma2_rn(e, pgB[P][1], vy);
                vz = __ffma2_rn(e, pgB[P][2], vz);
              }
              // dL/dx_c partial: sum e gB - sum w (x - z), gB = s2 gB'
              v[4 * cc + 0] = fmaf(vx.x + vx.y, s2, -(ux.x + ux.y));
              v[4 * cc + 1] = fmaf(vy.x + vy.y, s2, -(uy.x + uy.y));
              v[4 * cc + 2] = fmaf(vz.x + vz.y, s2, -(uz.x + uz.y));
            }
          }
          const float tot = reduce_scatter16(v);
          const int cc = (lane & 15) >> 2, comp = lane & 3;
          if (lane < 16 && c0 + cc < len)
            reinterpret_cast<float*>(px + (size_t)b2 * A.N + first + c0 + cc)[comp] = comp < 3 ? tot : 0.f;
        }
        __syncthreads();
        st = nst;
      }
      if (!ok) break;
      // dL/dz per row: sum over the warps, then over the slices, per row block
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int rb = 2 * b2 + hh;
        if (rb >= g.nblk) break;  // uniform
        float2 acc[kPairs][3];
#pragma unroll
        for (int kk = 0; kk < kPairs; ++kk)
#pragma unroll
          for (int a = 0; a < 3; ++a) acc[kk][a] = gz2[2 * hh + kk][a];
        float totz[3];
        reduce_warps<3>(sm, acc, totz);
        if (split_complete<3>(sm, g, rb, sl, (unsigned)(A.nsteps - 1 - k), A.part, A.cnt, totz)) {
          df vv[16];
#pragma unroll
          for (int q = 0; q < 16; ++q) vv[q] = df_make(0.f);
          const int r = rb * kBlockPts + tid;
          if (tid < kBlockPts && r < A.M) {
            const float4 y = ld_cg(A.rows + r);
            const float* rt = rtape + (size_t)r * 5;
            const float C = rt[0], lam = rt[1];
            const float uu[3] = {rt[2], rt[3], rt[4]};
            const float yy[3] = {y.x, y.y, y.z};
            // dL/dy = R^T dL/dz + lambda gP + gQ^T u
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
              for (int i = 0; i < 3; ++i)
                df_add(vv[12 + i], coef[1 + i] + coef[7 + i] * yy[0] + coef[10 + i] * yy[1] + coef[13 + i] * yy[2]);
            }
          }
          owned_block_sum<16>(vv, reinterpret_cast<df*>(sm.prep), recs + (size_t)rb * 16);
        }
      }
    }
    if (!ok || !grid_sync(A.ctl, epoch, G, A.timeout_ns, 102)) {
      ok = false;
      break;
    }
    // upstream gradient of the previous step's output pose, identical in every block
    reduce_block_partials<16>(recs, g.nblk, s_red, s_tot);
    if (tid < 12) s_g[tid] = df_val(s_tot[tid]);
    __syncthreads();
    const float gxb[3] = {df_val(s_tot[12]) / (float)A.N, df_val(s_tot[13]) / (float)A.N,
                          df_val(s_tot[14]) / (float)A.N};
    // dL/dx_c: this block's share of the columns, row-block partials in order
    for (int c = blockIdx.x * kThreads + tid; c < A.N; c += G * kThreads) {
      float sx = gxb[0], sy = gxb[1], sz = gxb[2];
      int b = 0;
      const int nb2 = (g.nblk + 1) / 2;
      for (; b + 16 <= nb2; b += 16) {  // 16 loads in flight, summed in order
        float4 p[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) p[j] = __ldcg(px + (size_t)(b + j) * A.N + c);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          sx += p[j].x;
          sy += p[j].y;
          sz += p[j].z;
        }
      }
      for (; b < nb2; ++b) {
        const float4 p = __ldcg(px + (size_t)b * A.N + c);
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
  SweepGeom geo;
  size_t smem;
};

AdjPlan plan_adj(int N, int M, int device) {
  AdjPlan P;
  P.smem = sizeof(AdjSmem);
  const int limit = persistent_grid_limit(device, (const void*)emicp_adjoint_kernel, P.smem);
  // units own pairs of row blocks: plan the slices for ceil(nblk / 2) owned blocks
  const int nblk = (M + kBlockPts - 1) / kBlockPts;
  const int nb2 = (nblk + 1) / 2;
  const SweepGeomH h = plan_sweep(nb2 * kBlockPts, N, limit);
  P.geo = SweepGeom{M, N, nblk, h.slices, h.slice_len, nb2 * h.slices};
  P.grid = P.geo.units < limit ? P.geo.units : limit;
  return P;
}

}  // namespace

// Workspace of the adjoint: control block and counters (cleared), gradient
// accumulators gX, gY (cleared), split partials, records and column partials.
size_t emicp_adjoint_ws_need(int N, int M, int device) {
  const AdjPlan P = plan_adj(N, M, device);
  Carve c(nullptr);
  c.take<Ctl>(1);
  c.take<unsigned>((size_t)P.geo.nblk);
  c.take<float4>((size_t)N);
  c.take<float4>((size_t)M);
  c.take<float>(12);
  c.take<float>((size_t)P.geo.nblk * P.geo.slices * 3 * kBlockPts);
  c.take<df>((size_t)2 * P.geo.nblk * 16);
  c.take<float4>((size_t)2 * ((P.geo.nblk + 1) / 2) * N);
  return c.off;
}

int enqueue_emicp_adjoint(const EmicpAdjointLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  const AdjPlan P = plan_adj(L.N, L.M, device);
  Carve c(ws);
  Ctl* ctl = c.take<Ctl>(1);
  unsigned* cnt = c.take<unsigned>((size_t)P.geo.nblk);
  float4* gX = c.take<float4>((size_t)L.N);
  float4* gY = c.take<float4>((size_t)L.M);
  float* g_in = c.take<float>(12);
  const size_t zero_bytes = c.off;
  float* part = c.take<float>((size_t)P.geo.nblk * P.geo.slices * 3 * kBlockPts);
  df* rec = c.take<df>((size_t)2 * P.geo.nblk * 16);
  float4* part_x = c.take<float4>((size_t)2 * ((P.geo.nblk + 1) / 2) * L.N);
  if (c.off > ws_bytes) return (int)cudaErrorInvalidValue;
  e = cudaMemsetAsync(ws, 0, zero_bytes, st);
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
  A.part = part;
  A.cnt = cnt;
  A.rec = rec;
  A.part_x = part_x;
  A.ctl = ctl;
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
