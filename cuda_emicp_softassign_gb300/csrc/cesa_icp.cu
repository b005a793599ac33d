// ICP for sm_103a: the iterations of icp() (src/icp.cpp:122-290) in one
// persistent cooperative launch.
//
// Reference iteration: every source point y is moved by the current pose,
// z = R y + t, and matched to its nearest target point x_nn; then
//   Xc = mean of the matches, S = sum (x_nn - Xc)(y - Yc)^T (Yc = mean of Y,
//   fixed), pose = findRTfromS(Xc, Yc, S).
// maxIteration iterations, no convergence test. The reference finds the
// matches with FLANN's randomised kd-trees and default search checks, which
// is approximate; here the search is exhaustive (exact nearest neighbour, the
// first of equal distances in X order), tiled over (row block, X slice) units:
//   phase A: a lane owns 4 moved source points (two packed pairs) and scans
//            an X slice staged through shared memory; per element the squared
//            distance by direct differences (3 FADD, FMUL + 2 FFMA, packed)
//            and a compare-select of (distance, index);
//   phase B: after a grid barrier, each row takes the first minimum over the
//            slices in slice order and adds its match to 16 compensated
//            moments (sum x, sum x (y - Yc)^T, sum (y - Yc), sum of distances);
//   after a second barrier every block reduces the moments in a fixed order
//   and solves Horn's pose (the same carried-eigenbasis solve as EM-ICP).
// Coordinates are centred by exact offsets before the loop (S is translation
// invariant; Xc, Yc and t are shifted back).
#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {
namespace {

constexpr int kIcpRows = kThreads * 4;  // source points per unit (4 per thread)
constexpr int kIcpTile = 1024;          // target points per shared-memory tile (16 KB)
constexpr int kIcpNV = 16;              // moments: sum x (3), sum x yd^T (9), sum yd (3), sum d2

struct IcpArgs {
  const float4* rows;  // Y' centred (M), moved by the pose
  const float4* cols;  // X' centred (N), searched
  int M, N, iters;
  int nrb, S, slice_len, units;
  const CenterHdr* hdr;
  float* dRt;          // PoseIO in/out, caller frame
  float2* part;        // [S][M]: (squared distance, index bits) per slice
  int* nn_out;         // optional [M]: the last iteration's matches
  df* rbpart;          // [2][grid][kIcpNV]
  Ctl* ctl;
  double* trace;
  int trace_cap;
  int* d_status;
  uint64_t timeout_ns;
};

__global__ void __launch_bounds__(kThreads, 2) icp_kernel(const IcpArgs A) {
  __shared__ float4 s_x[kIcpTile];
  __shared__ float s_pose[12];
  __shared__ float s_hdr[9];  // oX, oY, mean of Y'
  __shared__ df s_red[kThreads];
  __shared__ df s_tot[kIcpNV];
  __shared__ HornState<float> horn;  // carried eigenbasis (thread 0)

  const int tid = threadIdx.x;
  const unsigned G = gridDim.x;
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
  unsigned epoch = 0;
  bool ok = true;
  for (int iter = 0; iter < A.iters && ok; ++iter) {
    float R[9], tc[3];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
    // ---- phase A: per (row block, X slice), the first nearest point of each row
    for (int u = blockIdx.x; u < A.units; u += G) {
      const int rb = u / A.S, sl = u - rb * A.S;
      const int cb = sl * A.slice_len, ce = min(cb + A.slice_len, A.N);
      float2 q[2][3];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        float v[2][3];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          const int r = rb * kIcpRows + (2 * p + l) * kThreads + tid;
          const float4 y = r < A.M ? ld_cg(A.rows + r) : make_float4(0.f, 0.f, 0.f, 0.f);
          v[l][0] = -(R[0] * y.x + R[1] * y.y + R[2] * y.z + tc[0]);
          v[l][1] = -(R[3] * y.x + R[4] * y.y + R[5] * y.z + tc[1]);
          v[l][2] = -(R[6] * y.x + R[7] * y.y + R[8] * y.z + tc[2]);
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) q[p][d] = make_float2(v[0][d], v[1][d]);
      }
      float bd[2][2];
      int bi[2][2];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          bd[p][l] = __int_as_float(0x7f800000);  // +inf
          bi[p][l] = -1;
        }
      for (int j0 = cb; j0 < ce; j0 += kIcpTile) {
        const int n = min(kIcpTile, ce - j0);
        __syncthreads();
        for (int k = tid; k < n; k += kThreads) s_x[k] = ld_cg(A.cols + j0 + k);
        __syncthreads();
#pragma unroll 4
        for (int j = 0; j < n; ++j) {
          const float4 s = s_x[j];
#pragma unroll
          for (int p = 0; p < 2; ++p) {
            const float2 d2 = dist2_pair(q[p], s);
            if (d2.x < bd[p][0]) {
              bd[p][0] = d2.x;
              bi[p][0] = j0 + j;
            }
            if (d2.y < bd[p][1]) {
              bd[p][1] = d2.y;
              bi[p][1] = j0 + j;
            }
          }
        }
      }
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          const int r = rb * kIcpRows + (2 * p + l) * kThreads + tid;
          if (r < A.M) __stcg(A.part + (size_t)sl * A.M + r, make_float2(bd[p][l], __int_as_float(bi[p][l])));
        }
    }
    if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, 70)) {
      ok = false;
      break;
    }
    // ---- phase B: the first minimum over the slices, and the moments
    df* mom = A.rbpart + (size_t)(iter & 1) * G * kIcpNV;
    {
      df v[kIcpNV];
#pragma unroll
      for (int k = 0; k < kIcpNV; ++k) v[k] = df_make(0.f);
      for (int r = blockIdx.x * kThreads + tid; r < A.M; r += G * kThreads) {
        float best = __int_as_float(0x7f800000);
        int bi = 0;
        for (int s = 0; s < A.S; ++s) {
          const float2 p = __ldcg(A.part + (size_t)s * A.M + r);
          if (p.x < best) {
            best = p.x;
            bi = __float_as_int(p.y);
          }
        }
        if (A.nn_out) A.nn_out[r] = bi;
        const float4 x = ld_cg(A.cols + bi);
        const float4 y = ld_cg(A.rows + r);
        const float xv[3] = {x.x, x.y, x.z};
        const float yd[3] = {y.x - s_hdr[6], y.y - s_hdr[7], y.z - s_hdr[8]};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          df_add(v[i], xv[i]);
          df_add(v[12 + i], yd[i]);
#pragma unroll
          for (int j = 0; j < 3; ++j) df_add_prod(v[3 + i + 3 * j], xv[i], yd[j]);
        }
        df_add(v[15], best);
      }
      block_reduce_df<kIcpNV>(v, s_red);
      if (tid == 0)
#pragma unroll
        for (int k = 0; k < kIcpNV; ++k)
          __stcg(reinterpret_cast<float2*>(mom + (size_t)blockIdx.x * kIcpNV + k), make_float2(v[k].hi, v[k].lo));
    }
    if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, 72)) {
      ok = false;
      break;
    }
    // ---- the pose (every block computes the same one)
    reduce_block_partials<kIcpNV>(mom, (int)G, s_red, s_tot);
    if (tid == 0) {
      float Xc[3], Ym[3], S[9];
      for (int i = 0; i < 3; ++i) {
        Xc[i] = (float)(df_dbl(s_tot[i]) / (double)A.M);
        Ym[i] = s_hdr[6 + i];
      }
      // S = sum (x - Xc)(y - Yc)^T = sum x yd^T - Xc (sum yd)^T
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          df a = s_tot[3 + i + 3 * j];
          df_add_prod(a, -Xc[i], df_val(s_tot[12 + j]));
          S[i + 3 * j] = df_val(a);
        }
      float q[4], gap = 0.f, lmax = 0.f, Rn[9], tn[3];
      horn_quaternion<float>(S, horn, q, &gap, &lmax);
      quat_to_pose<float>(q, Xc, Ym, Rn, tn);  // centred frame: t' = Xc' - R Ym
      for (int k = 0; k < 9; ++k) s_pose[k] = Rn[k];
      for (int k = 0; k < 3; ++k) s_pose[9 + k] = tn[k];
      if (blockIdx.x == 0) {
        if (A.trace && iter < A.trace_cap) {
          double* rec = A.trace + (size_t)iter * 32;
          float to[3];
          pose_from_centred(Rn, tn, &s_hdr[0], &s_hdr[3], to);
          rec[0] = iter;
          rec[1] = iter;
          rec[2] = df_dbl(s_tot[15]);
          for (int i = 0; i < 3; ++i) {
            rec[3 + i] = (double)Xc[i] + s_hdr[i];
            rec[6 + i] = (double)Ym[i] + s_hdr[3 + i];
            rec[27 + i] = to[i];
          }
          for (int k = 0; k < 9; ++k) {
            rec[9 + k] = S[k];
            rec[18 + k] = Rn[k];
          }
          rec[30] = gap;
          rec[31] = lmax;
        }
        A.ctl->steps_done = iter + 1;
      }
    }
    __syncthreads();
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

struct IcpPlan {
  int grid, nrb, S, slice_len, units;
};

// Row blocks of kIcpRows source points and X slices of at least 256 points,
// as many slices as fill whole waves of the co-resident grid best (up to 4).
IcpPlan plan_icp(int N, int M, int device) {
  IcpPlan P;
  const int limit = persistent_grid_limit(device, (const void*)icp_kernel, 0);
  P.nrb = (M + kIcpRows - 1) / kIcpRows;
  const int max_s = (N + 255) / 256;
  int bestS = 1;
  double best = -1.0;
  for (int w = 1; w <= 4; ++w) {
    int S = (w * limit) / P.nrb;
    if (S < 1) S = 1;
    if (S > max_s) S = max_s;
    const int units = P.nrb * S;
    const int waves = (units + limit - 1) / limit;
    const double eff = (double)units / ((double)waves * limit);
    if (eff > best + 0.02) {
      best = eff;
      bestS = S;
    }
  }
  P.slice_len = (N + bestS - 1) / bestS;
  P.S = (N + P.slice_len - 1) / P.slice_len;
  P.units = P.nrb * P.S;
  P.grid = P.units < limit ? P.units : limit;
  return P;
}

struct IcpCarved {
  Ctl* ctl;
  CenterHdr* hdr;
  float4* rows;
  float4* cols;
  float2* part;
  df* rbpart;
};

IcpCarved carve_icp(void* base, const IcpPlan& P, int N, int M, size_t* total) {
  Carve c(base);
  IcpCarved w;
  w.ctl = c.take<Ctl>(1);
  w.hdr = c.take<CenterHdr>(1);
  w.rows = c.take<float4>((size_t)M);
  w.cols = c.take<float4>((size_t)N);
  w.part = c.take<float2>((size_t)P.S * M);
  w.rbpart = c.take<df>((size_t)2 * P.grid * kIcpNV);
  if (total) *total = c.off;
  return w;
}

}  // namespace

size_t icp_ws_need(int N, int M, int device) {
  const IcpPlan P = plan_icp(N, M, device);
  size_t total = 0;
  carve_icp(nullptr, P, N, M, &total);
  return total;
}

int enqueue_icp(const IcpLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  const IcpPlan P = plan_icp(L.N, L.M, device);
  size_t total = 0;
  IcpCarved w = carve_icp(ws, P, L.N, L.M, &total);
  if (total > ws_bytes) return (int)cudaErrorInvalidValue;
  if (grid_used) *grid_used = P.grid;
  e = cudaMemsetAsync(w.ctl, 0, sizeof(Ctl), st);
  if (e != cudaSuccess) return (int)e;
  prep_center_kernel<<<1, 1024, 0, st>>>(L.dX, L.N, L.dY, L.M, w.hdr);
  const int pb = 256, pg_x = (L.N + pb - 1) / pb, pg_y = (L.M + pb - 1) / pb;
  prep_pack_kernel<<<pg_x < 1024 ? pg_x : 1024, pb, 0, st>>>(L.dX, L.N, w.hdr, 0, 0.f, w.cols);
  prep_pack_kernel<<<pg_y < 1024 ? pg_y : 1024, pb, 0, st>>>(L.dY, L.M, w.hdr, 1, 0.f, w.rows);
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (L.iters <= 0) return 0;
  IcpArgs A;
  A.rows = w.rows;
  A.cols = w.cols;
  A.M = L.M;
  A.N = L.N;
  A.iters = L.iters;
  A.nrb = P.nrb;
  A.S = P.S;
  A.slice_len = P.slice_len;
  A.units = P.units;
  A.hdr = w.hdr;
  A.dRt = L.dRt;
  A.part = w.part;
  A.nn_out = L.nn_out;
  A.rbpart = w.rbpart;
  A.ctl = w.ctl;
  A.trace = L.trace;
  A.trace_cap = L.trace_cap;
  A.d_status = L.d_status;
  A.timeout_ns = L.timeout_ns;
  void* args[] = {(void*)&A};
  return (int)cudaLaunchCooperativeKernel((const void*)icp_kernel, dim3(P.grid), dim3(kThreads), args, 0, st);
}

}  // namespace cesa
