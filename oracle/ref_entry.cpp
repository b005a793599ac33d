/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * C entry points into the reference's own CPU code, compiled unmodified from
 * the reference tree (src/emicp_cpu.cpp, src/findRTfromS.cpp,
 * src/cloud2data.cpp) by oracle/build.py into oracle/_ref/libref_emicp.so.
 *
 *   ref_emicp_cpu      -> emicp_cpu()    src/emicp_cpu.cpp:186-547
 *   ref_find_rt_from_s -> findRTfromS()  src/findRTfromS.cpp:33-97
 *
 * Point sets are passed as SoA float arrays [x0..xn-1, y0.., z0..] like the
 * reference's cloud2data() output (src/cloud2data.cpp:29-46).
 */
#include <cstdio>
#include <fcntl.h>
#include <unistd.h>
#include "3dregistration.h"

static pcl::PointCloud<pcl::PointXYZ>::Ptr soa_to_cloud(const float* p, int n) {
  pcl::PointCloud<pcl::PointXYZ>::Ptr c(new pcl::PointCloud<pcl::PointXYZ>);
  for (int i = 0; i < n; ++i) c->push_back(pcl::PointXYZ(p[i], p[n + i], p[2 * n + i]));
  return c;
}

extern "C" int ref_emicp_cpu(const float* X, int N, const float* Y, int M, float* R, float* t,
                             float sigma_p2, float sigma_inf, float sigma_factor, float d_02,
                             int quiet) {
  registrationParameters param;
  param.JMAX = 0; param.I0 = 0; param.I1 = 0;
  param.alpha = 0.f; param.T_0 = 0.f; param.TFACTOR = 0.f; param.moutlier = 0.f;
  param.sigma_p2 = sigma_p2; param.sigma_inf = sigma_inf;
  param.sigma_factor = sigma_factor; param.d_02 = d_02;
  param.maxIteration = 0;
  param.noviewer = 1; param.nostop = 1; param.notimer = 1;
  param.argc = 0; param.argv = nullptr;
  pcl::PointCloud<pcl::PointXYZ>::Ptr cx = soa_to_cloud(X, N);
  pcl::PointCloud<pcl::PointXYZ>::Ptr cy = soa_to_cloud(Y, M);
  /* the reference prints one line per sigma step on stderr */
  int saved = -1;
  if (quiet) {
    fflush(stderr);
    saved = dup(2);
    int devnull = open("/dev/null", O_WRONLY);
    if (devnull >= 0) { dup2(devnull, 2); close(devnull); }
  }
  emicp_cpu(cx, cy, R, t, param);
  if (saved >= 0) { fflush(stderr); dup2(saved, 2); close(saved); }
  return 0;
}

extern "C" void ref_find_rt_from_s(const float* Xc, const float* Yc, const float* S, float* R,
                                   float* t) {
  findRTfromS(Xc, Yc, S, R, t);
}
