// Softassign for sm_103a: the whole annealing schedule of softassign()
// (src/softassign.cu:486-822) in one persistent cooperative launch.
//
// Reference inner iteration (src/softassign.cu:494-798). Rows r are X points
// (N), columns c are Y points (M):
//   M_rc = exp(-(|x_r - (R y_c + t)|^2 - alpha)/T) / sqrt(T)          (updateM)
//   I1 times:  rs = M 1 + s;  M_r. /= rs_r;  s /= rs                   (row pass, slack s)
//              cs = M^T 1 + u; M_.c /= cs_c; u /= cs                   (column pass, slack u)
//   w = M 1 (no slack), sumM = sum w, Xw = w .* X, Yw = cs .* Y (last cs, before
//   its normalisation), Xc = sum Xw / sumM, Yc = sum Yw / sumM,
//   Xw -= Xc, Yw -= Yc, S = Xw^T (M Yw), pose = findRTfromS(Xc, Yc, S)
// s and u persist across all inner iterations (src/softassign.cu:385-390).
//
// Matrix-free form: M_rc = K_rc a_r b_c. K is recomputed in every sweep and
// never stored. Row sweeps own 128 X points and stream Y. Column sweeps own
// 128 Y points and stream X. Each sweep element costs 3 FADD + FMUL + 2 FFMA
// (direct-difference d^2), 1 FFMA (exponent), 1 MUFU ex2 and 1 FFMA (weighted
// sum): 7 FP32 ops + 1 MUFU op. Per pose update there are 2*I1 + 1 sweeps and
// 2*I1 + 1 grid barriers.
//
// The reference's S is not translation invariant, because X is weighted and
// only then centred. Coordinates are centred on the device for accuracy, and
// the original-frame S is rebuilt exactly from 32 compensated sums of
// centred-frame per-row and per-column quantities.
#include "cesa_kernels.h"
#include "cesa_pose.h"
#include "cesa_prep.cuh"
#include "cesa_sweep.cuh"

namespace cesa {

constexpr int kSaNV = 32;

struct SoftArgs {
  float4* rows;    // X' centred, .w = a_r   (N)
  float4* cols;    // Y' centred, .w = b_c   (M)
  float4* colfin;  // per column (g y', g), g = b_c cs_c after the last column pass
  float* s;        // slack column [N]
  float* u;        // slack row [M]
  float* rs;       // last row sums incl. slack [N]
  float* cs;       // last column sums incl. slack [M]
  float* w_out;    // optional [N]
  int N, M;
  SweepGeom gr, gc;  // row sweeps (own X, stream Y) / column sweeps (own Y, stream X)
  int JMAX, I0, I1;
  float alpha, T0, TFACTOR;
  const CenterHdr* hdr;
  float* dRt;
  float* part_r;
  unsigned* cnt_r;
  float* part_c;
  unsigned* cnt_c;
  df* bpart;  // [2][grid][kSaNV]
  Ctl* ctl;
  double* trace;
  int trace_cap;
  int* d_status;
  uint64_t timeout_ns;
};

// Streamed Y columns for row sweeps: (R y' + t', b_c) with b_c := 1 in the
// first pass of an inner iteration.
struct RowPrep {
  float R[9], tc[3];
  bool unit_w;
  __device__ __forceinline__ const float4* operator()(SweepSmem& sm, int stage, int len) const {
    for (int c = threadIdx.x; c < len; c += kThreads) {
      const float4 y = sm.raw[stage][c];
      sm.prep[c] = make_float4(R[0] * y.x + R[1] * y.y + R[2] * y.z + tc[0],
                               R[3] * y.x + R[4] * y.y + R[5] * y.z + tc[1],
                               R[6] * y.x + R[7] * y.y + R[8] * y.z + tc[2], unit_w ? 1.f : y.w);
    }
    __syncthreads();
    return sm.prep;
  }
};

// Sinkhorn sweep element: acc += K * weight(streamed).
struct SinkElem {
  float nk, c0;  // K = 2^(c0 + nk d^2)
  __device__ __forceinline__ void operator()(float (&acc)[1], const float (&p)[3], float4 s,
                                             float4) const {
    const float dx = s.x - p[0];
    const float dy = s.y - p[1];
    const float dz = s.z - p[2];
    float d2 = dx * dx;
    d2 = fmaf(dy, dy, d2);
    d2 = fmaf(dz, dz, d2);
    const float e = ex2_approx(fmaf(d2, nk, c0));
    acc[0] = fmaf(e, s.w, acc[0]);
  }
};

// Final row sweep element: w += K b, m += K g, V' += K g y'.
struct FinalElem {
  float nk, c0;
  __device__ __forceinline__ void operator()(float (&acc)[5], const float (&p)[3], float4 s,
                                             float4 hg) const {
    const float dx = s.x - p[0];
    const float dy = s.y - p[1];
    const float dz = s.z - p[2];
    float d2 = dx * dx;
    d2 = fmaf(dy, dy, d2);
    d2 = fmaf(dz, dz, d2);
    const float e = ex2_approx(fmaf(d2, nk, c0));
    acc[0] = fmaf(e, s.w, acc[0]);
    acc[1] = fmaf(e, hg.w, acc[1]);
    acc[2] = fmaf(e, hg.x, acc[2]);
    acc[3] = fmaf(e, hg.y, acc[3]);
    acc[4] = fmaf(e, hg.z, acc[4]);
  }
};

// Row pass finalize (normalizeMbySinkhorn_row + Saxpy, src/softassign.cu:538-561).
struct RowFin {
  float4* rows;
  float* s;
  float* rs;
  int N;
  bool first;
  __device__ void operator()(int blk, const float (&tot)[1]) const {
    const int r = blk * kBlockPts + (int)threadIdx.x;
    if (threadIdx.x < kBlockPts && r < N) {
      const float a_old = first ? 1.f : __ldcg(&rows[r].w);
      const float s_old = __ldcg(&s[r]);
      const float sum = fmaf(a_old, tot[0], s_old);
      __stcg(&rows[r].w, a_old / sum);
      __stcg(&s[r], s_old / sum);
      __stcg(&rs[r], sum);
    }
  }
};

// Column pass finalize (normalizeMbySinkhorn_col + Saxpy, src/softassign.cu:579-597).
// On the last pass also records (g y', g) and the column moments for Yc.
struct ColFin {
  float4* cols;
  float4* colfin;
  float* u;
  float* cs;
  int M;
  bool first, last;
  df* red;
  df* acc;  // block accumulator slots 28..31
  __device__ void operator()(int blk, const float (&tot)[1]) const {
    df v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = df_make(0.f);
    const int c = blk * kBlockPts + (int)threadIdx.x;
    if (threadIdx.x < kBlockPts && c < M) {
      const float4 y = __ldcg(&cols[c]);
      const float b_old = first ? 1.f : y.w;
      const float u_old = __ldcg(&u[c]);
      const float sum = fmaf(b_old, tot[0], u_old);
      const float b_new = b_old / sum;
      __stcg(&cols[c].w, b_new);
      __stcg(&u[c], u_old / sum);
      __stcg(&cs[c], sum);
      if (last) {
        const float g = b_new * sum;
        __stcg(&colfin[c], make_float4(g * y.x, g * y.y, g * y.z, g));
        df_add(v[0], sum);
        df_add_prod(v[1], sum, y.x);
        df_add_prod(v[2], sum, y.y);
        df_add_prod(v[3], sum, y.z);
      }
    }
    if (last) block_accumulate<4>(v, red, acc);
  }
};

// Final row finalize: w, m, V' and the 28 row-side moments.
//  0: sum w        1-3: sum w x'         4-12: sum w x'_i V'_j (i + 3j)
// 13-15: sum w^2 x'  16-18: sum V'        19-21: sum m w x'   22: sum m
// 23-25: sum w V'    26: sum w^2         27: sum w m
struct FinalFin {
  const float4* rows;
  float* w_out;
  int N;
  df* red;
  df* acc;
  __device__ void operator()(int blk, const float (&tot)[5]) const {
    df v[28];
#pragma unroll
    for (int k = 0; k < 28; ++k) v[k] = df_make(0.f);
    const int r = blk * kBlockPts + (int)threadIdx.x;
    if (threadIdx.x < kBlockPts && r < N) {
      const float4 x = __ldcg(&rows[r]);
      const float a = x.w;
      const float w = a * tot[0], m = a * tot[1];
      const float V[3] = {a * tot[2], a * tot[3], a * tot[4]};
      const float xp[3] = {x.x, x.y, x.z};
      if (w_out) w_out[r] = w;
      const float w2 = w * w, mw = m * w;
      df_add(v[0], w);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        df_add_prod(v[1 + i], w, xp[i]);
        const float wx = w * xp[i];
#pragma unroll
        for (int j = 0; j < 3; ++j) df_add_prod(v[4 + i + 3 * j], wx, V[j]);
        df_add_prod(v[13 + i], w2, xp[i]);
        df_add(v[16 + i], V[i]);
        df_add_prod(v[19 + i], mw, xp[i]);
        df_add_prod(v[23 + i], w, V[i]);
      }
      df_add(v[22], m);
      df_add_prod(v[26], w, w);
      df_add_prod(v[27], w, m);
    }
    block_accumulate<28>(v, red, acc);
  }
};

// df helpers for the (thread 0) moment assembly
__device__ __forceinline__ df dmul(df a, float b) {  // (a.hi + a.lo) * b, ~df precision
  df r = df_make(0.f);
  df_add_prod(r, a.hi, b);
  r.lo = __fmaf_rn(a.lo, b, r.lo);
  return r;
}

__global__ void __launch_bounds__(kThreads, 2) softassign_kernel(const SoftArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SweepSmem& sm = *reinterpret_cast<SweepSmem*>(smem_raw);
  __shared__ float s_pose[12];
  __shared__ df s_acc[kSaNV];
  __shared__ df s_red[kThreads];
  __shared__ df s_tot[kSaNV];
  __shared__ float s_hdr[8];

  const int tid = threadIdx.x;
  const unsigned G = gridDim.x;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&sm.full[s], 1);
    mbar_init_fence();
    for (int k = 0; k < 3; ++k) {
      s_hdr[k] = A.hdr->oX[k];
      s_hdr[3 + k] = A.hdr->oY[k];
    }
    float R[9], t[3], tc[3];
    for (int k = 0; k < 9; ++k) R[k] = A.dRt[k];
    for (int k = 0; k < 3; ++k) t[k] = A.dRt[9 + k];
    pose_to_centred(R, t, &s_hdr[0], &s_hdr[3], tc);
    for (int k = 0; k < 9; ++k) s_pose[k] = R[k];
    for (int k = 0; k < 3; ++k) s_pose[9 + k] = tc[k];
  }
  __syncthreads();

  HornState<float> horn;
  horn.reset();
  Pipe pipe;
  pipe_init(pipe);
  unsigned epoch = 0, round_r = 0, round_c = 0;
  const StreamSrc src_cols{A.cols, nullptr, false};
  const StreamSrc src_rows{A.rows, nullptr, false};
  const StreamSrc src_final{A.cols, A.colfin, false};
  float T = A.T0;
  int step = 0;
  bool ok = true;

  for (int Titer = 0; Titer < A.JMAX && ok; ++Titer) {
    // K = exp((alpha - d^2)/T) / sqrt(T) = 2^(c0 + nk d^2)
    const float kk = kLog2e / T;
    const float nk = -kk;
    const float c0 = fmaf(A.alpha, kk, -0.5f * log2f(T));
    for (int iter0 = 0; iter0 < A.I0 && ok; ++iter0, ++step) {
      if (tid < kSaNV) s_acc[tid] = df_make(0.f);
      float R[9], tc[3];
#pragma unroll
      for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
      __syncthreads();
      const SinkElem se{nk, c0};
      for (int k = 0; k < A.I1 && ok; ++k) {
        // row pass: own X rows, stream transformed Y columns weighted by b
        RowPrep rp;
#pragma unroll
        for (int q = 0; q < 9; ++q) rp.R[q] = R[q];
#pragma unroll
        for (int q = 0; q < 3; ++q) rp.tc[q] = tc[q];
        rp.unit_w = (k == 0);
        const RowFin rf{A.rows, A.s, A.rs, A.N, k == 0};
        ok = sweep_units<1>(sm, pipe, A.gr, src_cols, A.rows, false, R, tc, round_r++, A.part_r,
                            A.cnt_r, se, rp, rf, A.ctl, A.timeout_ns, 30) &&
             grid_sync(A.ctl, epoch, G, A.timeout_ns, 32);
        if (!ok) break;
        // column pass: own transformed Y columns, stream X rows weighted by a
        const ColFin cf{A.cols, A.colfin, A.u, A.cs, A.M, k == 0, k == A.I1 - 1, s_red, s_acc + 28};
        ok = sweep_units<1>(sm, pipe, A.gc, src_rows, A.cols, true, R, tc, round_c++, A.part_c,
                            A.cnt_c, se, NoPrep{}, cf, A.ctl, A.timeout_ns, 40) &&
             grid_sync(A.ctl, epoch, G, A.timeout_ns, 42);
      }
      if (!ok) break;
      // final row sweep: w, m, V'
      {
        RowPrep rp;
#pragma unroll
        for (int q = 0; q < 9; ++q) rp.R[q] = R[q];
#pragma unroll
        for (int q = 0; q < 3; ++q) rp.tc[q] = tc[q];
        rp.unit_w = false;
        const FinalElem fe{nk, c0};
        const FinalFin ff{A.rows, A.w_out, A.N, s_red, s_acc};
        ok = sweep_units<5>(sm, pipe, A.gr, src_final, A.rows, false, R, tc, round_r++, A.part_r,
                            A.cnt_r, fe, rp, ff, A.ctl, A.timeout_ns, 50);
        if (!ok) break;
      }
      df* bp = A.bpart + (size_t)(step & 1) * G * kSaNV;
      if (tid < kSaNV) {
        const df a = s_acc[tid];
        __stcg(reinterpret_cast<float2*>(bp + (size_t)blockIdx.x * kSaNV + tid),
               make_float2(a.hi, a.lo));
      }
      ok = grid_sync(A.ctl, epoch, G, A.timeout_ns, 52);
      if (!ok) break;
      reduce_block_partials<kSaNV>(bp, (int)G, s_red, s_tot);
      if (tid == 0) {
        const float* oX = &s_hdr[0];
        const float* oY = &s_hdr[3];
        const df A1 = s_tot[0];
        const float sumM = df_val(A1);
        const float inv = 1.f / sumM;
        float Xcp[3], Ycp[3];
        for (int i = 0; i < 3; ++i) {
          Xcp[i] = df_val(s_tot[1 + i]) * inv;
          Ycp[i] = df_val(s_tot[29 + i]) * inv;
        }
        const float rho = df_val(s_tot[28]) * inv;
        const float C5 = df_val(s_tot[22]);
        const float C7 = df_val(s_tot[26]);
        // P_i = C4_i - rho C2_i - Xc'_i C5 + rho Xc'_i A1
        // Q_j = C6_j - C3_j - Yc'_j C7 + Yc'_j A1
        // Z   = C8 - rho C7 - C5 + rho A1
        float P[3], Q[3];
        for (int i = 0; i < 3; ++i) {
          df p = s_tot[19 + i];
          df_add(p, dmul(s_tot[13 + i], -rho));
          df_add_prod(p, -Xcp[i], C5);
          df_add(p, dmul(A1, rho * Xcp[i]));
          P[i] = df_val(p);
          df q = s_tot[23 + i];
          df_add(q, df{-s_tot[16 + i].hi, -s_tot[16 + i].lo});
          df_add_prod(q, -Ycp[i], C7);
          df_add(q, dmul(A1, Ycp[i]));
          Q[i] = df_val(q);
        }
        df z = s_tot[27];
        df_add(z, dmul(s_tot[26], -rho));
        df_add(z, df{-s_tot[22].hi, -s_tot[22].lo});
        df_add(z, dmul(A1, rho));
        const float Z = df_val(z);
        // S_ij = C1_ij - C2_i Yc'_j - Xc'_i C3_j + Xc'_i Yc'_j A1
        //        + P_i oY_j + oX_i Q_j + oX_i oY_j Z
        float S[9];
        for (int j = 0; j < 3; ++j)
          for (int i = 0; i < 3; ++i) {
            df sij = s_tot[4 + i + 3 * j];
            df_add(sij, dmul(s_tot[13 + i], -Ycp[j]));
            df_add(sij, dmul(s_tot[16 + j], -Xcp[i]));
            df_add(sij, dmul(A1, Xcp[i] * Ycp[j]));
            df_add_prod(sij, P[i], oY[j]);
            df_add_prod(sij, oX[i], Q[j]);
            df_add_prod(sij, oX[i] * oY[j], Z);
            S[i + 3 * j] = df_val(sij);
          }
        float Xc[3], Yc[3], Yd[3];
        for (int i = 0; i < 3; ++i) {
          Xc[i] = Xcp[i] + oX[i];
          df y = df_make(Ycp[i]);
          df_add_prod(y, rho, oY[i]);
          Yc[i] = df_val(y);
          df yd = df_make(Ycp[i]);
          df_add_prod(yd, rho - 1.f, oY[i]);
          Yd[i] = df_val(yd);  // Yc - oY
        }
        float q[4], gap = 0.f, lmax = 0.f, Rn[9], tn[3];
        horn_quaternion<float>(S, horn, q, &gap, &lmax);
        // centred-frame translation t' = Xc' - R (Yc - oY)
        quat_to_pose<float>(q, Xcp, Yd, Rn, tn);
        for (int k = 0; k < 9; ++k) s_pose[k] = Rn[k];
        for (int k = 0; k < 3; ++k) s_pose[9 + k] = tn[k];
        if (blockIdx.x == 0) {
          if (A.trace && step < A.trace_cap) {
            double* rec = A.trace + (size_t)step * 32;
            float to[3];
            pose_from_centred(Rn, tn, oX, oY, to);
            rec[0] = step;
            rec[1] = T;
            rec[2] = df_dbl(A1);
            for (int i = 0; i < 3; ++i) {
              rec[3 + i] = Xc[i];
              rec[6 + i] = Yc[i];
              rec[27 + i] = to[i];
            }
            for (int k = 0; k < 9; ++k) {
              rec[9 + k] = S[k];
              rec[18 + k] = Rn[k];
            }
            rec[30] = gap;
            rec[31] = lmax;
          }
          A.ctl->steps_done = step + 1;
        }
      }
      __syncthreads();
    }
    T = T * A.TFACTOR;  // FP32, src/softassign.cu:820
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
  }
}

// ------------------------------------------------------------------ host side
namespace {
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

struct SaPlan {
  int grid;
  SweepGeom gr, gc;
  size_t smem;
};

SaPlan plan_sa(int N, int M, int device) {
  SaPlan P;
  P.smem = sizeof(SweepSmem);
  const int limit = persistent_grid_limit(device, (const void*)softassign_kernel, P.smem);
  const SweepGeomH r = plan_sweep(N, M, limit);
  const SweepGeomH c = plan_sweep(M, N, limit);
  P.gr = SweepGeom{r.n_own, r.n_stream, r.nblk, r.slices, r.slice_len, r.units};
  P.gc = SweepGeom{c.n_own, c.n_stream, c.nblk, c.slices, c.slice_len, c.units};
  const int mu = r.units > c.units ? r.units : c.units;
  P.grid = mu < limit ? mu : limit;
  return P;
}

struct SaCarved {
  Ctl* ctl;
  unsigned* cnt_r;
  unsigned* cnt_c;
  CenterHdr* hdr;
  float4* rows;
  float4* cols;
  float4* colfin;
  float *s, *u, *rs, *cs;
  float* part_r;
  float* part_c;
  df* bpart;
};

SaCarved carve_sa(void* base, const SaPlan& P, int N, int M, size_t* total) {
  Carve c(base);
  SaCarved w;
  w.ctl = c.take<Ctl>(1);
  w.cnt_r = c.take<unsigned>((size_t)P.gr.nblk);
  w.cnt_c = c.take<unsigned>((size_t)P.gc.nblk);
  w.hdr = c.take<CenterHdr>(1);
  w.rows = c.take<float4>((size_t)N);
  w.cols = c.take<float4>((size_t)M);
  w.colfin = c.take<float4>((size_t)M);
  w.s = c.take<float>((size_t)N);
  w.u = c.take<float>((size_t)M);
  w.rs = c.take<float>((size_t)N);
  w.cs = c.take<float>((size_t)M);
  w.part_r = c.take<float>((size_t)P.gr.units * 5 * kBlockPts);
  w.part_c = c.take<float>((size_t)P.gc.units * 1 * kBlockPts);
  w.bpart = c.take<df>((size_t)2 * P.grid * kSaNV);
  if (total) *total = c.off;
  return w;
}
}  // namespace

size_t softassign_ws_need(int N, int M, int form, int device) {
  (void)form;
  const SaPlan P = plan_sa(N, M, device);
  size_t total = 0;
  carve_sa(nullptr, P, N, M, &total);
  return total;
}

int enqueue_softassign(const SoftassignLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st,
                       int* grid_used) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  const SaPlan P = plan_sa(L.N, L.M, device);
  size_t total = 0;
  SaCarved w = carve_sa(ws, P, L.N, L.M, &total);
  if (total > ws_bytes) return (int)cudaErrorInvalidValue;
  if (grid_used) *grid_used = P.grid;
  e = cudaMemsetAsync(w.ctl, 0, sizeof(Ctl), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.cnt_r, 0, sizeof(unsigned) * (size_t)P.gr.nblk, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.cnt_c, 0, sizeof(unsigned) * (size_t)P.gc.nblk, st);
  if (e != cudaSuccess) return (int)e;
  prep_center_kernel<<<1, 1024, 0, st>>>(L.dX, L.N, L.dY, L.M, w.hdr);
  const int pb = 256, pg_x = (L.N + pb - 1) / pb, pg_y = (L.M + pb - 1) / pb;
  prep_pack_kernel<<<pg_x < 1024 ? pg_x : 1024, pb, 0, st>>>(L.dX, L.N, w.hdr, 0, 1.f, w.rows);
  prep_pack_kernel<<<pg_y < 1024 ? pg_y : 1024, pb, 0, st>>>(L.dY, L.M, w.hdr, 1, 1.f, w.cols);
  if (L.s_io)
    e = cudaMemcpyAsync(w.s, L.s_io, sizeof(float) * (size_t)L.N, cudaMemcpyDeviceToDevice, st);
  else
    fill_kernel<<<pg_x < 1024 ? pg_x : 1024, pb, 0, st>>>(w.s, L.N, L.moutlier);
  if (e == cudaSuccess && L.u_io)
    e = cudaMemcpyAsync(w.u, L.u_io, sizeof(float) * (size_t)L.M, cudaMemcpyDeviceToDevice, st);
  else if (e == cudaSuccess)
    fill_kernel<<<pg_y < 1024 ? pg_y : 1024, pb, 0, st>>>(w.u, L.M, L.moutlier);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (L.JMAX <= 0 || L.I0 <= 0) return 0;

  SoftArgs A;
  A.rows = w.rows;
  A.cols = w.cols;
  A.colfin = w.colfin;
  A.s = w.s;
  A.u = w.u;
  A.rs = w.rs;
  A.cs = w.cs;
  A.w_out = L.w_out;
  A.N = L.N;
  A.M = L.M;
  A.gr = P.gr;
  A.gc = P.gc;
  A.JMAX = L.JMAX;
  A.I0 = L.I0;
  A.I1 = L.I1;
  A.alpha = L.alpha;
  A.T0 = L.T_0;
  A.TFACTOR = L.TFACTOR;
  A.hdr = w.hdr;
  A.dRt = L.dRt;
  A.part_r = w.part_r;
  A.cnt_r = w.cnt_r;
  A.part_c = w.part_c;
  A.cnt_c = w.cnt_c;
  A.bpart = w.bpart;
  A.ctl = w.ctl;
  A.trace = L.trace;
  A.trace_cap = L.trace_cap;
  A.d_status = L.d_status;
  A.timeout_ns = L.timeout_ns;
  void* args[] = {(void*)&A};
  e = cudaLaunchCooperativeKernel((const void*)softassign_kernel, dim3(P.grid), dim3(kThreads), args,
                                  P.smem, st);
  if (e != cudaSuccess) return (int)e;
  // optional vector outputs
  if (L.s_io) e = cudaMemcpyAsync(L.s_io, w.s, sizeof(float) * (size_t)L.N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && L.u_io)
    e = cudaMemcpyAsync(L.u_io, w.u, sizeof(float) * (size_t)L.M, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && L.rs_out)
    e = cudaMemcpyAsync(L.rs_out, w.rs, sizeof(float) * (size_t)L.N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && L.cs_out)
    e = cudaMemcpyAsync(L.cs_out, w.cs, sizeof(float) * (size_t)L.M, cudaMemcpyDeviceToDevice, st);
  return (int)e;
}

}  // namespace cesa
