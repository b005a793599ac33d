// Preparation kernels and frame helpers shared by the registration kernels.
//
// Centring: the mean of each cloud is taken with compensated (df) sums and
// rounded to an FP32 offset o; the kernels then work on x - o. The pose
// enters and leaves in the caller's frame, and the translation is converted
// with compensated arithmetic, so large coordinate offsets (scanner frames)
// cost no precision in the N x M loops.
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

static __global__ void prep_center_kernel(const float* __restrict__ X, int N, const float* __restrict__ Y,
                                   int M, CenterHdr* hdr) {
  // One block: means of X and Y in df, rounded to float; then mean of X - oX.
  __shared__ df red[6 * (1024 / 32)];
  __shared__ float s_o[6];
  df v[6];
  for (int k = 0; k < 6; ++k) v[k] = df_make(0.f);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    df_add(v[0], X[i]);
    df_add(v[1], X[N + i]);
    df_add(v[2], X[2 * N + i]);
  }
  for (int i = threadIdx.x; i < M; i += blockDim.x) {
    df_add(v[3], Y[i]);
    df_add(v[4], Y[M + i]);
    df_add(v[5], Y[2 * M + i]);
  }
  block_reduce_df<6>(v, red);
  if (threadIdx.x == 0) {
    for (int k = 0; k < 3; ++k) s_o[k] = (float)(df_dbl(v[k]) / (double)N);
    for (int k = 0; k < 3; ++k) s_o[3 + k] = (float)(df_dbl(v[3 + k]) / (double)M);
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
