// cesa_register: the reference's registration command line (src/main.cpp:232-499)
// over libcesa.so, headless. Same flags, defaults and R, t file format:
//
//   cesa_register -pointFileX=<ply|txt> -pointFileY=<ply|txt>
//                 [-softassign (default) | -emicp | -icp | -emicpcpu]
//                 [-JMAX= -I0= -I1= -alpha= -T_0= -TFACTOR= -moutlier=]
//                 [-sigma_p2= -sigma_inf= -sigma_factor= -d_02=] [-maxIteration=]
//                 [-alignScaleOnce] [-pointsReductionRate= | -pointsReductionRateX= -pointsReductionRateY=]
//                 [-loadRTfromFile=] [-saveRTtoFile=] [-noviewer -nostop -notimer]
//
// Solves min ||X - (R Y + t)||. Additions (no counterpart in the reference):
// -seed= (pointsReduction's seed; the reference seeds with the clock) and
// -sinkhorn_form=auto|matrix_free|materialised|banded. There is no viewer: the
// viewer flags are accepted and have no effect. -emicpcpu runs the GPU EM-ICP
// (this build has no CPU registration path) and says so on stderr.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cesa.h"

namespace {

// -name or --name, optionally followed by =value
const char* find_arg(int argc, char** argv, const char* name) {
  const size_t n = std::strlen(name);
  for (int i = 1; i < argc; ++i) {
    const char* a = argv[i];
    while (*a == '-') ++a;
    if (a == argv[i]) continue;
    if (std::strncmp(a, name, n) == 0 && (a[n] == '\0' || a[n] == '=')) return a + n;
  }
  return nullptr;
}

bool flag(int argc, char** argv, const char* name) { return find_arg(argc, argv, name) != nullptr; }

bool str_arg(int argc, char** argv, const char* name, std::string& out) {
  const char* v = find_arg(argc, argv, name);
  if (!v || *v != '=') return false;
  out = v + 1;
  return true;
}

// 0 when absent or unparsable, as the reference's getCmdLineArgumentInt/Float
int int_arg(int argc, char** argv, const char* name) {
  std::string s;
  return str_arg(argc, argv, name, s) ? std::atoi(s.c_str()) : 0;
}
float float_arg(int argc, char** argv, const char* name) {
  std::string s;
  return str_arg(argc, argv, name, s) ? (float)std::atof(s.c_str()) : 0.f;
}

void print_rt(const float* R, const float* t) {
  std::printf("R\n");
  for (int r = 0; r < 9; ++r) {
    std::printf("%f ", R[r]);
    if ((r + 1) % 3 == 0) std::printf("\n");
  }
  std::printf("t\n");
  for (int r = 0; r < 3; ++r) std::printf("%f ", t[r]);
  std::printf("\n");
}

std::vector<float> to_soa(const float* xyz, int n) {
  std::vector<float> s(3 * (size_t)n);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) s[(size_t)k * n + i] = xyz[3 * i + k];
  return s;
}

}  // namespace

int main(int argc, char** argv) {
  std::string fx, fy;
  if (!str_arg(argc, argv, "pointFileX", fx) || !str_arg(argc, argv, "pointFileY", fy)) {
    std::fprintf(stderr, "Wrong arguments: -pointFileX=<file> -pointFileY=<file> are required.\n");
    std::fprintf(stderr, "min ||X - (R*Y+t) ||\n");
    return 1;
  }
  std::printf("option: pointFileX= %s\noption: pointFileY=%s\n", fx.c_str(), fy.c_str());
  const bool is_icp = flag(argc, argv, "icp");
  const bool is_emicp = flag(argc, argv, "emicp");
  const bool is_emicp_cpu = flag(argc, argv, "emicpcpu");
  bool is_sa = flag(argc, argv, "softassign");
  if (!is_icp && !is_emicp && !is_emicp_cpu && !is_sa) is_sa = true;  // default algorithm

  cesa_params p;
  cesa_params_default(&p);
  if (is_sa) {
    if (int v = int_arg(argc, argv, "JMAX")) p.JMAX = v;
    if (int v = int_arg(argc, argv, "I0")) p.I0 = v;
    if (int v = int_arg(argc, argv, "I1")) p.I1 = v;
    if (float v = float_arg(argc, argv, "alpha")) p.alpha = v;
    if (float v = float_arg(argc, argv, "T_0")) p.T_0 = v;
    if (float v = float_arg(argc, argv, "TFACTOR")) p.TFACTOR = v;
    const float mo = float_arg(argc, argv, "moutlier");
    p.moutlier = mo ? mo : (float)(1 / sqrtf(p.T_0) * expf(-1.0f));
    std::printf("softassgin paramters\nJMAX %d\nI0 %d\nI1 %d\nalpha %g\nT_0 %g\nTFACTOR %g\nmoutlier %g\n", p.JMAX,
                p.I0, p.I1, p.alpha, p.T_0, p.TFACTOR, p.moutlier);
  }
  if (is_icp) {
    if (int v = int_arg(argc, argv, "maxIteration")) p.maxIteration = v;
    std::printf("ICP paramters\nmaxIteration %d\n", p.maxIteration);
  }
  if (is_emicp || is_emicp_cpu) {
    if (float v = float_arg(argc, argv, "sigma_p2")) p.sigma_p2 = v;
    if (float v = float_arg(argc, argv, "sigma_inf")) p.sigma_inf = v;
    if (float v = float_arg(argc, argv, "sigma_factor")) p.sigma_factor = v;
    if (float v = float_arg(argc, argv, "d_02")) p.d_02 = v;
    std::printf("EM-ICP paramters\nsigma_p2 %g\nsigma_inf %g\nsigma_factor %g\nd_02 %g\n", p.sigma_p2, p.sigma_inf,
                p.sigma_factor, p.d_02);
  }
  std::string form;
  if (str_arg(argc, argv, "sinkhorn_form", form)) {
    if (form == "matrix_free") p.sinkhorn_form = CESA_SINKHORN_MATRIX_FREE;
    else if (form == "materialised") p.sinkhorn_form = CESA_SINKHORN_MATERIALISED;
    else if (form == "banded") p.sinkhorn_form = CESA_SINKHORN_BANDED;
    else p.sinkhorn_form = CESA_SINKHORN_AUTO;
  }
  const unsigned long long seed = (unsigned long long)int_arg(argc, argv, "seed");

  float* X = nullptr;
  float* Y = nullptr;
  int nx = 0, ny = 0;
  int rc = cesa_load_points(fx.c_str(), &X, &nx);
  if (rc == CESA_OK) rc = cesa_load_points(fy.c_str(), &Y, &ny);
  if (rc != CESA_OK) {
    std::fprintf(stderr, "loadFile failed: %s\n", cesa_status_string(rc));
    cesa_free(X);
    cesa_free(Y);
    return 1;
  }
  if (flag(argc, argv, "alignScaleOnce")) {
    rc = cesa_align_scale_once(X, nx, Y, ny);
    if (rc != CESA_OK) std::fprintf(stderr, "alignScaleOnce: %s\n", cesa_status_string(rc));
  }
  float rate = float_arg(argc, argv, "pointsReductionRate");
  if (rate) {
    cesa_points_reduction(X, &nx, rate, seed);
    cesa_points_reduction(Y, &ny, rate, seed + 1);
    std::printf("number of points X,Y are reduced to %g%% of original.\n", rate);
  } else {
    if ((rate = float_arg(argc, argv, "pointsReductionRateX"))) {
      cesa_points_reduction(X, &nx, rate, seed);
      std::printf("number of points X are reduced to %g%% of original.\n", rate);
    }
    if ((rate = float_arg(argc, argv, "pointsReductionRateY"))) {
      cesa_points_reduction(Y, &ny, rate, seed + 1);
      std::printf("number of points Y are reduced to %g%% of original.\n", rate);
    }
  }
  std::printf("Xsize: %d\nYsize: %d\n", nx, ny);

  float R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, t[3] = {0, 0, 0};
  std::string rt_in;
  if (str_arg(argc, argv, "loadRTfromFile", rt_in) && cesa_load_rt(rt_in.c_str(), R, t) != CESA_OK) {
    std::fprintf(stderr, "Fail to read RT from file [%s]\n", rt_in.c_str());
    return 1;
  }
  print_rt(R, t);
  const std::vector<float> xs = to_soa(X, nx), ys = to_soa(Y, ny);
  cesa_free(X);
  cesa_free(Y);
  if (is_emicp_cpu)
    std::fprintf(stderr, "-emicpcpu: this build has no CPU registration path; running EM-ICP on the GPU\n");
  const auto t0 = std::chrono::steady_clock::now();
  if (is_icp) rc = cesa_icp(xs.data(), nx, ys.data(), ny, R, t, &p, nullptr);
  if (rc == CESA_OK && (is_emicp || is_emicp_cpu)) rc = cesa_emicp(xs.data(), nx, ys.data(), ny, R, t, &p, nullptr);
  if (rc == CESA_OK && is_sa) rc = cesa_softassign(xs.data(), nx, ys.data(), ny, R, t, &p, nullptr);
  const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rc != CESA_OK) std::fprintf(stderr, "registration: %s\n", cesa_status_string(rc));
  std::printf("elapsed %f\n", el);
  print_rt(R, t);
  std::string rt_out;
  if (str_arg(argc, argv, "saveRTtoFile", rt_out)) cesa_save_rt(rt_out.c_str(), R, t);
  return rc == CESA_OK ? 0 : 1;
}
