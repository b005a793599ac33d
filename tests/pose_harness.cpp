// Host build of the device pose solver (cesa_pose.h) for CPU tests.
#include "cesa_pose.h"

extern "C" {
// Solves K consecutive S matrices (K x 9, h_S layout) with one warm-started
// state, as the persistent kernels do; q_out: K x 4, gap_out: K.
int pose_sequence_f32(const float* S, int K, float* q_out, float* gap_out) {
  cesa::HornState<float> st;
  st.reset();
  int fallbacks = 0;
  for (int k = 0; k < K; ++k) {
    float q[4], gap = 0.f, lmax = 0.f;
    fallbacks += cesa::horn_quaternion<float>(S + 9 * k, st, q, &gap, &lmax);
    for (int i = 0; i < 4; ++i) q_out[4 * k + i] = q[i];
    gap_out[k] = gap;
  }
  return fallbacks;
}
// The same with the plain kernels' solver (certified inverse iteration, Jacobi
// fallback); returns the number of solves that fell back to Jacobi.
int pose_sequence_fast_f32(const float* S, int K, float* q_out, float* lmax_out) {
  cesa::HornState<float> st;
  st.reset();
  int jacobi = 0;
  for (int k = 0; k < K; ++k) {
    float q[4], gap = 0.f, lmax = 0.f;
    cesa::horn_quaternion_fast<float>(S + 9 * k, st, q, &gap, &lmax);
    jacobi += gap >= 0.f;
    for (int i = 0; i < 4; ++i) q_out[4 * k + i] = q[i];
    lmax_out[k] = lmax;
  }
  return jacobi;
}
int pose_sequence_f64(const double* S, int K, double* q_out, double* gap_out) {
  cesa::HornState<double> st;
  st.reset();
  int fallbacks = 0;
  for (int k = 0; k < K; ++k) {
    double q[4], gap = 0, lmax = 0;
    fallbacks += cesa::horn_quaternion<double>(S + 9 * k, st, q, &gap, &lmax);
    for (int i = 0; i < 4; ++i) q_out[4 * k + i] = q[i];
    gap_out[k] = gap;
  }
  return fallbacks;
}
}
