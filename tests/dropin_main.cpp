// A user program written against the reference API (src/3dregistration.h):
// reads SoA clouds from argv files, runs emicp(), emicp_cpu(), softassign() or
// icp() with the reference defaults, prints R (row-major) and t. The mode
// "printRT" runs emicp() and prints the pose with the API's printRT() instead.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "3dregistration.h"

static pcl::PointCloud<pcl::PointXYZ>::Ptr load(const char* path) {
  FILE* f = std::fopen(path, "rb");
  pcl::PointCloud<pcl::PointXYZ>::Ptr c(new pcl::PointCloud<pcl::PointXYZ>);
  if (!f) return c;
  int n = 0;
  if (std::fread(&n, sizeof(int), 1, f) != 1) n = 0;
  std::vector<float> v(3 * static_cast<size_t>(n));
  if (n > 0 && std::fread(v.data(), sizeof(float), v.size(), f) != v.size()) n = 0;
  std::fclose(f);
  for (int i = 0; i < n; ++i) c->push_back(pcl::PointXYZ(v[3 * i], v[3 * i + 1], v[3 * i + 2]));
  return c;
}

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  registrationParameters param;
  param.JMAX = 100; param.I0 = 5; param.I1 = 3; param.alpha = 3.0f; param.T_0 = 100.0f;
  param.TFACTOR = 0.95f; param.moutlier = (float)(1 / sqrtf(param.T_0) * expf(-1.0f));
  param.sigma_p2 = 0.01f; param.sigma_inf = 0.00001f; param.sigma_factor = 0.9f; param.d_02 = 0.01f;
  param.maxIteration = 30; param.noviewer = 1; param.nostop = 1; param.notimer = 1;
  param.argc = argc; param.argv = argv;
  if (argc > 4) param.JMAX = std::atoi(argv[4]);
  float h_R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, h_t[3] = {0, 0, 0};
  pcl::PointCloud<pcl::PointXYZ>::Ptr X = load(argv[2]), Y = load(argv[3]);
  if (std::strcmp(argv[1], "printRT") == 0) {
    emicp(X, Y, h_R, h_t, param);
    printRT(h_R, h_t);
    return 0;
  }
  if (std::strcmp(argv[1], "emicp") == 0)
    emicp(X, Y, h_R, h_t, param);
  else if (std::strcmp(argv[1], "emicp_cpu") == 0)
    emicp_cpu(X, Y, h_R, h_t, param);
  else if (std::strcmp(argv[1], "icp") == 0)
    icp(X, Y, h_R, h_t, param);
  else
    softassign(X, Y, h_R, h_t, param);
  // cloud2data and findRTfromS are part of the same API
  float* soa = nullptr;
  int n = 0;
  cloud2data(X, &soa, n);
  int ok = (n == (int)X->size()) && (n == 0 || soa[0] == X->points[0].x);
  delete[] soa;
  for (int i = 0; i < 9; ++i) std::printf("%.9g ", h_R[i]);
  for (int i = 0; i < 3; ++i) std::printf("%.9g ", h_t[i]);
  std::printf("%d\n", ok);
  return 0;
}
