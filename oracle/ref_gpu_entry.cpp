/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * C entry points into the reference's own GPU registration code, whose CUDA
 * kernels and cuBLAS calls run on the host under oracle/emu (oracle/build.py
 * builds oracle/_ref/libref_gpu.so from the reference sources, with only their
 * kernel-launch syntax rewritten):
 *
 *   ref_softassign -> softassign()  src/softassign.cu:256-886
 *   ref_emicp_gpu  -> emicp()       src/emicp.cu:247-716
 *
 * The link wraps the reference's findRTfromS() (src/findRTfromS.cpp:33-97,
 * called once per pose update at src/softassign.cu:787 and src/emicp.cu:633):
 * the wrapper records the update's Xc, Yc, S and the pose it returns, so a
 * caller gets the reference's own per-update trace. Record layout (doubles, 32
 * per update):
 *   [0] update  [1] 0 (the caller fills T or sigma_p2)  [2] 0  [3..5] Xc
 *   [6..8] Yc  [9..17] S (h_S layout)  [18..26] R row-major  [27..29] t
 * Point sets are SoA float arrays [x0..xn-1, y0.., z0..] (src/cloud2data.cpp:29-46).
 */
#include <fcntl.h>
#include <unistd.h>

#include <cstdio>
#include <cstring>

#include "3dregistration.h"

namespace {
double* g_trace = nullptr;
int g_trace_cap = 0;
int g_trace_n = 0;

pcl::PointCloud<pcl::PointXYZ>::Ptr soa_to_cloud(const float* p, int n) {
  pcl::PointCloud<pcl::PointXYZ>::Ptr c(new pcl::PointCloud<pcl::PointXYZ>);
  for (int i = 0; i < n; ++i) c->push_back(pcl::PointXYZ(p[i], p[n + i], p[2 * n + i]));
  return c;
}
}  // namespace

// The reference's findRTfromS, reached through the linker's --wrap of its
// mangled name (CESA_FIND_RT_WRAP / CESA_FIND_RT_REAL are set by the build).
extern "C" void CESA_FIND_RT_REAL(const float* Xc, const float* Yc, const float* S, float* R, float* t);
extern "C" void CESA_FIND_RT_WRAP(const float* Xc, const float* Yc, const float* S, float* R, float* t) {
  CESA_FIND_RT_REAL(Xc, Yc, S, R, t);
  if (g_trace && g_trace_n < g_trace_cap) {
    double* r = g_trace + 32 * (size_t)g_trace_n;
    memset(r, 0, 32 * sizeof(double));
    r[0] = g_trace_n;
    for (int k = 0; k < 3; ++k) {
      r[3 + k] = Xc[k];
      r[6 + k] = Yc[k];
      r[27 + k] = t[k];
    }
    for (int k = 0; k < 9; ++k) {
      r[9 + k] = S[k];
      r[18 + k] = R[k];
    }
  }
  ++g_trace_n;
}

extern "C" int ref_softassign(const float* X, int N, const float* Y, int M, float* R, float* t, int JMAX, int I0,
                              int I1, float alpha, float T_0, float TFACTOR, float moutlier, double* trace,
                              int trace_cap, int quiet) {
  registrationParameters param;
  param.JMAX = JMAX;
  param.I0 = I0;
  param.I1 = I1;
  param.alpha = alpha;
  param.T_0 = T_0;
  param.TFACTOR = TFACTOR;
  param.moutlier = moutlier;
  param.sigma_p2 = 0.f;
  param.sigma_inf = 0.f;
  param.sigma_factor = 0.f;
  param.d_02 = 0.f;
  param.maxIteration = 0;
  param.noviewer = 1;
  param.nostop = 1;
  param.notimer = 1;
  param.argc = 0;
  param.argv = nullptr;
  pcl::PointCloud<pcl::PointXYZ>::Ptr cx = soa_to_cloud(X, N);
  pcl::PointCloud<pcl::PointXYZ>::Ptr cy = soa_to_cloud(Y, M);
  g_trace = trace;
  g_trace_cap = trace ? trace_cap : 0;
  g_trace_n = 0;
  // the reference prints one line per temperature on stderr
  int saved = -1;
  if (quiet) {
    fflush(stderr);
    saved = dup(2);
    int devnull = open("/dev/null", O_WRONLY);
    if (devnull >= 0) {
      dup2(devnull, 2);
      close(devnull);
    }
  }
  softassign(cx, cy, R, t, param);
  if (saved >= 0) {
    fflush(stderr);
    dup2(saved, 2);
    close(saved);
  }
  const int n = g_trace_n;
  g_trace = nullptr;
  return n;
}

extern "C" int ref_emicp_gpu(const float* X, int N, const float* Y, int M, float* R, float* t, float sigma_p2,
                             float sigma_inf, float sigma_factor, float d_02, double* trace, int trace_cap,
                             int quiet) {
  registrationParameters param;
  param.JMAX = 0;
  param.I0 = 0;
  param.I1 = 0;
  param.alpha = 0.f;
  param.T_0 = 0.f;
  param.TFACTOR = 0.f;
  param.moutlier = 0.f;
  param.sigma_p2 = sigma_p2;
  param.sigma_inf = sigma_inf;
  param.sigma_factor = sigma_factor;
  param.d_02 = d_02;
  param.maxIteration = 0;
  param.noviewer = 1;
  param.nostop = 1;
  param.notimer = 1;
  param.argc = 0;
  param.argv = nullptr;
  pcl::PointCloud<pcl::PointXYZ>::Ptr cx = soa_to_cloud(X, N);
  pcl::PointCloud<pcl::PointXYZ>::Ptr cy = soa_to_cloud(Y, M);
  g_trace = trace;
  g_trace_cap = trace ? trace_cap : 0;
  g_trace_n = 0;
  int saved = -1;
  if (quiet) {
    fflush(stderr);
    saved = dup(2);
    int devnull = open("/dev/null", O_WRONLY);
    if (devnull >= 0) {
      dup2(devnull, 2);
      close(devnull);
    }
  }
  emicp(cx, cy, R, t, param);
  if (saved >= 0) {
    fflush(stderr);
    dup2(saved, 2);
    close(saved);
  }
  const int n = g_trace_n;
  g_trace = nullptr;
  return n;
}
