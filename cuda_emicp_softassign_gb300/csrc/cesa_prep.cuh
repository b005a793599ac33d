// Preparation kernels and frame helpers shared by the registration kernels.
//
// Centring: each cloud is shifted by an offset o chosen so that x - o is
// exact in FP32 (see exact_offset). The pose enters and leaves in the
// caller's frame, and the translation is converted with compensated
// arithmetic, so large coordinate offsets (scanner frames) cost no precision
// in the N x M loops.
#pragma once
#include "cesa_common.cuh"
#include "cesa_kernels.h"

namespace cesa {

// t' = t + R oY - oX (caller frame -> centred frame), compensated.
__device__ __forceinline__ void pose_to_centred(const float R[9], const float t[3], const float oX[3],
                                const float oY[3], float tc[3]) {
  for (int i = 0; i < 3; ++i) {
    df a = df_make(t[i]);
    for (int j = 0; j < 3; ++j) df_add_prod(a, R[3 * i + j], oY[j]);
    df_add(a, -oX[i]);
    tc[i] = df_val(a);
  }
}
// t = t' + oX - R oY
__device__ __forceinline__ void pose_from_centred(const float R[9], const float tc[3], const float oX[3],
                                  const float oY[3], float t[3]) {
  for (int i = 0; i < 3; ++i) {
    df a = df_make(tc[i]);
    df_add(a, oX[i]);
    for (int j = 0; j < 3; ++j) df_add_prod(a, -R[3 * i + j], oY[j]);
    t[i] = df_val(a);
  }
}

// Exact centring offsets. For each axis of a cloud: q = 2^ceil(log2(extent)),
// o = round(mean / q) * q when |mean| >= 4 q, else 0. Every point then lies
// within 1.5 q of o while |x| >= 2.5 q, so x - o is exact in FP32: centring
// removes a scanner-frame offset without rounding a single coordinate, and
// data that straddles the origin is left untouched.
__device__ __forceinline__ float exact_offset(double mean, float lo, float hi) {
  const float ext = hi - lo;
  if (!(ext > 0.f)) return 0.f;
  const float q = exp2f(ceilf(log2f(ext)));
  if (fabs(mean) < 4.0 * (double)q) return 0.f;
  return (float)(rint(mean / (double)q) * (double)q);
}

// One block of up to 1024 threads: means (df) and extents of X and Y, exact
// offsets, and the means of the centred clouds (EM-ICP rows with C_r <= 1e-6
// use mean(X'); the Softassign final sweep centres its Y moments on mean(Y')).
__device__ __forceinline__ void center_block(const float* __restrict__ X, int N, const float* __restrict__ Y,
                                             int M, CenterHdr* hdr) {
  __shared__ df red[6 * (1024 / 32)];
  __shared__ float s_lo[12][32], s_hi[12][32];
  __shared__ float s_o[6];
  df v[6];
  float lo[6], hi[6];
  for (int k = 0; k < 6; ++k) {
    v[k] = df_make(0.f);
    lo[k] = 3.0e38f;
    hi[k] = -3.0e38f;
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const float x = X[k * N + i];
      df_add(v[k], x);
      lo[k] = fminf(lo[k], x);
      hi[k] = fmaxf(hi[k], x);
    }
  for (int i = threadIdx.x; i < M; i += blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const float y = Y[k * M + i];
      df_add(v[3 + k], y);
      lo[3 + k] = fminf(lo[3 + k], y);
      hi[3 + k] = fmaxf(hi[3 + k], y);
    }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < 6; ++k)
    for (int off = 16; off > 0; off >>= 1) {
      lo[k] = fminf(lo[k], __shfl_down_sync(0xffffffffu, lo[k], off));
      hi[k] = fmaxf(hi[k], __shfl_down_sync(0xffffffffu, hi[k], off));
    }
  if (lane == 0)
    for (int k = 0; k < 6; ++k) {
      s_lo[k][warp] = lo[k];
      s_hi[k][warp] = hi[k];
    }
  block_reduce_df<6>(v, red);
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int k = 0; k < 6; ++k) {
      float l = s_lo[k][0], h = s_hi[k][0];
      for (int w = 1; w < nw; ++w) {
        l = fminf(l, s_lo[k][w]);
        h = fmaxf(h, s_hi[k][w]);
      }
      const double mean = df_dbl(v[k]) / (double)(k < 3 ? N : M);
      s_o[k] = exact_offset(mean, l, h);
    }
  }
  __syncthreads();
  df w[6];
  for (int k = 0; k < 6; ++k) w[k] = df_make(0.f);
  for (int i = threadIdx.x; i < N; i += blockDim.x)
    for (int k = 0; k < 3; ++k) df_add(w[k], __fsub_rn(X[k * N + i], s_o[k]));
  for (int i = threadIdx.x; i < M; i += blockDim.x)
    for (int k = 0; k < 3; ++k) df_add(w[3 + k], __fsub_rn(Y[k * M + i], s_o[3 + k]));
  block_reduce_df<6>(w, red);
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; ++k) {
      hdr->oX[k] = s_o[k];
      hdr->oY[k] = s_o[3 + k];
      hdr->xmean[k] = (float)(df_dbl(w[k]) / (double)N);
      hdr->ymean[k] = (float)(df_dbl(w[3 + k]) / (double)M);
    }
    hdr->oX[3] = hdr->oY[3] = hdr->xmean[3] = hdr->ymean[3] = 0.f;
  }
}

static __global__ void __launch_bounds__(1024) prep_center_kernel(const float* __restrict__ X, int N, const float* __restrict__ Y,
                                          int M, CenterHdr* hdr) {
  center_block(X, N, Y, M, hdr);
}

// SoA -> centred float4 (x - o, w0).
static __global__ void prep_pack_kernel(const float* __restrict__ P, int n, const CenterHdr* hdr, int which,
                                 float w0, float4* __restrict__ out) {
  const float* o = which == 0 ? hdr->oX : hdr->oY;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = make_float4(__fsub_rn(P[i], o[0]), __fsub_rn(P[n + i], o[1]),
                         __fsub_rn(P[2 * n + i], o[2]), w0);
}

static __global__ void fill_kernel(float* p, int n, float v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace cesa
