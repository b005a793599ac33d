// C++ drop-in layer: emicp(), softassign(), emicp_cpu(), icp(), findRTfromS(),
// printRT() and cloud2data() with the reference's signatures
// (src/3dregistration.h:82-116), implemented
// over the C ABI of libcesa.so. Compile this file into the program (as the
// reference README asks for emicp.cu / softassign.cu) and link -lcesa.
#include <atomic>
#include <cstdio>
#include <vector>

#include "3dregistration.h"
#include "cesa.h"

namespace {

void to_cesa(const registrationParameters& rp, cesa_params* p) {
  cesa_params_default(p);
  p->JMAX = rp.JMAX;
  p->I0 = rp.I0;
  p->I1 = rp.I1;
  p->alpha = rp.alpha;
  p->T_0 = rp.T_0;
  p->TFACTOR = rp.TFACTOR;
  p->moutlier = rp.moutlier;
  p->sigma_p2 = rp.sigma_p2;
  p->sigma_inf = rp.sigma_inf;
  p->sigma_factor = rp.sigma_factor;
  p->d_02 = rp.d_02;
  p->maxIteration = rp.maxIteration;
}

void soa(const pcl::PointCloud<pcl::PointXYZ>::Ptr& cloud, std::vector<float>& out) {
  const int n = static_cast<int>(cloud->size());
  out.resize(3 * static_cast<size_t>(n));
  for (int i = 0; i < n; ++i) {
    out[i] = cloud->points[i].x;
    out[n + i] = cloud->points[i].y;
    out[2 * n + i] = cloud->points[i].z;
  }
}

template <class Fn>
void run(const char* name, Fn fn, const pcl::PointCloud<pcl::PointXYZ>::Ptr& target,
         const pcl::PointCloud<pcl::PointXYZ>::Ptr& source, float* h_R, float* h_t,
         const registrationParameters& param) {
  if (!target || !source || !h_R || !h_t) {
    std::fprintf(stderr, "%s: %s\n", name, cesa_status_string(CESA_ERR_INVALID_ARGUMENT));
    return;
  }
  std::vector<float> X, Y;
  soa(target, X);
  soa(source, Y);
  cesa_params p;
  to_cesa(param, &p);
  const int rc = fn(X.data(), static_cast<int>(target->size()), Y.data(),
                    static_cast<int>(source->size()), h_R, h_t, &p, nullptr);
  if (rc != CESA_OK) std::fprintf(stderr, "%s: %s\n", name, cesa_status_string(rc));
}

}  // namespace

void emicp(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target,
           const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source, float* h_R, float* h_t,
           const registrationParameters& param) {
  run("emicp", cesa_emicp, cloud_target, cloud_source, h_R, h_t, param);
}

void emicp_cpu(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target,
               const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source, float* h_R, float* h_t,
               const registrationParameters& param) {
  // There is no CPU registration path in this library (a CPU fallback would
  // hide a missing GPU); the reference CLI's -emicpcpu flag is handled alike.
  static std::atomic<bool> noted{false};
  if (!noted.exchange(true))
    std::fprintf(stderr, "emicp_cpu: runs the GPU EM-ICP (this library has no CPU registration path)\n");
  run("emicp_cpu", cesa_emicp, cloud_target, cloud_source, h_R, h_t, param);
}

void icp(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target,
         const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source, float* h_R, float* h_t,
         const registrationParameters& param) {
  run("icp", cesa_icp, cloud_target, cloud_source, h_R, h_t, param);
}

void softassign(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_target,
                const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud_source, float* h_R, float* h_t,
                const registrationParameters& param) {
  run("softassign", cesa_softassign, cloud_target, cloud_source, h_R, h_t, param);
}

void findRTfromS(const float* h_Xc, const float* h_Yc, const float* h_S, float* h_R, float* h_t) {
  // per-thread fallback quaternion (the reference keeps one static q_pre,
  // src/findRTfromS.cpp:110)
  thread_local float q_pre[4] = {1.f, 0.f, 0.f, 0.f};
  cesa_find_rt_from_s(h_Xc, h_Yc, h_S, h_R, h_t, q_pre);
}

void printRT(const float* R, const float* t) {
  std::printf("R\n");
  for (int i = 0; i < 3; ++i) std::printf("%f %f %f \n", R[3 * i], R[3 * i + 1], R[3 * i + 2]);
  std::printf("t\n%f %f %f \n", t[0], t[1], t[2]);
}

void cloud2data(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud, float** X, int& Xsize) {
  Xsize = static_cast<int>(cloud->size());
  float* h = new float[3 * static_cast<size_t>(Xsize)];
  for (int i = 0; i < Xsize; ++i) {
    h[i] = cloud->points[i].x;
    h[Xsize + i] = cloud->points[i].y;
    h[2 * Xsize + i] = cloud->points[i].z;
  }
  *X = h;
}

void cloud2data(const pcl::PointCloud<pcl::PointXYZ>::Ptr cloud, boost::shared_array<float>& X,
                int& Xsize) {
  float* h = nullptr;
  cloud2data(cloud, &h, Xsize);
  X.reset(h);
}
