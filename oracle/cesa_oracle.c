/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's soft-correspondence registration path,
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker; the product (cuda_emicp_softassign_gb300/) never links it.
 *
 *   oracle_find_rt_from_s       findRTfromS + eigenvectorOfN,
 *                               src/findRTfromS.cpp:33-159 (Horn's quaternion
 *                               method); the LAPACK dsyev_ call is replaced by
 *                               a cyclic Jacobi eigen-solver written here.
 *   oracle_emicp_{f64,f32}      emicp_cpu(), src/emicp_cpu.cpp:186-547
 *                               (== emicp(), src/emicp.cu:247-716)
 *   oracle_softassign_{f64,f32} softassign(), src/softassign.cu:256-886
 *   *_step                      one annealing step with intermediates exposed
 *
 * Pinning: oracle_emicp_f64 and oracle_find_rt_from_s are checked against the
 * reference's own emicp_cpu()/findRTfromS() built from the reference sources
 * (oracle/_ref, see build.py) and against golden vectors generated from that
 * build (tests/golden/). The reference has no CPU Softassign; its restatement
 * follows src/softassign.cu line by line and is pinned through the shared
 * pose solver and the Sinkhorn invariants checked in tests/.
 */
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_TRACE_STRIDE 32

/*
 * Cyclic Jacobi eigen-decomposition of a symmetric 4x4 matrix (double).
 * On return A is diagonal (eigenvalues on the diagonal) and the columns of V
 * are the eigenvectors: A_in = V diag(A) V^T.
 */
static void jacobi4(double A[4][4], double V[4][4]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0, diag = 0;
    for (int p = 0; p < 4; ++p) {
      diag += A[p][p] * A[p][p];
      for (int q = p + 1; q < 4; ++q) off += A[p][q] * A[p][q];
    }
    if (off == 0.0 || off <= 1e-34 * diag) break;
    for (int p = 0; p < 3; ++p) {
      for (int q = p + 1; q < 4; ++q) {
        double apq = A[p][q];
        if (apq == 0.0) continue;
        double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
        double tt;
        if (fabs(theta) > 1e150)
          tt = 0.5 / theta;
        else
          tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(tt * tt + 1.0);
        double s = tt * c;
        for (int k = 0; k < 4; ++k) {
          double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 4; ++k) {
          double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 4; ++k) {
          double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
    }
  }
}

/*
 * findRTfromS, src/findRTfromS.cpp:33-97, in FP64.
 * S uses the reference's h_S layout (S[i+3j], read as Sxx=S[0], Sxy=S[1], ...).
 * q_prev (in/out, may be NULL) replaces the reference's static q_pre: if the
 * eigen-solve yields a non-finite vector the previous quaternion is reused
 * (src/findRTfromS.cpp:137-145). gap/lmax (may be NULL) report the relative
 * eigen-gap (l1 - l2)/max(|l1|, tiny) and the largest eigenvalue of N.
 * Returns 0, or 1 when the fallback quaternion was used.
 */
int oracle_find_rt_from_s(const double Xc[3], const double Yc[3], const double S[9], double R[9],
                          double t[3], double q_prev[4], double* gap, double* lmax) {
  const double Sxx = S[0], Sxy = S[1], Sxz = S[2];
  const double Syx = S[3], Syy = S[4], Syz = S[5];
  const double Szx = S[6], Szy = S[7], Szz = S[8];
  /* Horn's symmetric 4x4 N, src/findRTfromS.cpp:59-74 */
  double A[4][4] = {
      {Sxx + Syy + Szz, Syz - Szy, Szx - Sxz, Sxy - Syx},
      {Syz - Szy, Sxx - Syy - Szz, Sxy + Syx, Szx + Sxz},
      {Szx - Sxz, Sxy + Syx, Syy - Sxx - Szz, Syz + Szy},
      {Sxy - Syx, Szx + Sxz, Syz + Szy, Szz - Sxx - Syy},
  };
  double V[4][4];
  int finite = 1;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      if (!isfinite(A[i][j])) finite = 0;
  double q[4] = {1, 0, 0, 0};
  int used_prev = 0;
  if (finite) {
    jacobi4(A, V);
    int imax = 0;
    for (int i = 1; i < 4; ++i)
      if (A[i][i] > A[imax][imax]) imax = i;
    double l1 = A[imax][imax], l2 = -INFINITY;
    for (int i = 0; i < 4; ++i)
      if (i != imax && A[i][i] > l2) l2 = A[i][i];
    double nrm = 0;
    for (int i = 0; i < 4; ++i) nrm += V[i][imax] * V[i][imax];
    nrm = sqrt(nrm);
    for (int i = 0; i < 4; ++i) q[i] = V[i][imax] / nrm;
    if (gap) *gap = (l1 - l2) / fmax(fabs(l1), 1e-300);
    if (lmax) *lmax = l1;
  } else {
    used_prev = 1;
    if (gap) *gap = 0;
    if (lmax) *lmax = NAN;
  }
  for (int i = 0; i < 4; ++i)
    if (!isfinite(q[i])) used_prev = 1;
  if (used_prev) {
    if (q_prev)
      for (int i = 0; i < 4; ++i) q[i] = q_prev[i];
  } else if (q_prev) {
    for (int i = 0; i < 4; ++i) q_prev[i] = q[i];
  }
  const double q0 = q[0], qx = q[1], qy = q[2], qz = q[3];
  /* quaternion to rotation, src/findRTfromS.cpp:83-91 */
  R[0] = q0 * q0 + qx * qx - qy * qy - qz * qz;
  R[1] = 2 * (qx * qy - q0 * qz);
  R[2] = 2 * (qx * qz + q0 * qy);
  R[3] = 2 * (qy * qx + q0 * qz);
  R[4] = q0 * q0 - qx * qx + qy * qy - qz * qz;
  R[5] = 2 * (qy * qz - q0 * qx);
  R[6] = 2 * (qz * qx - q0 * qy);
  R[7] = 2 * (qz * qy + q0 * qx);
  R[8] = q0 * q0 - qx * qx - qy * qy + qz * qz;
  /* src/findRTfromS.cpp:94-96 */
  for (int i = 0; i < 3; ++i)
    t[i] = Xc[i] - (R[3 * i] * Yc[0] + R[3 * i + 1] * Yc[1] + R[3 * i + 2] * Yc[2]);
  return used_prev;
}

/* Eigen-decomposition exposed for tests: vals[4] ascending, vecs column-major 4x4. */
void oracle_eig4(const double N[16], double vals[4], double vecs[16]) {
  double A[4][4], V[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) A[i][j] = N[i + 4 * j];
  jacobi4(A, V);
  int idx[4] = {0, 1, 2, 3};
  for (int i = 0; i < 4; ++i)
    for (int j = i + 1; j < 4; ++j)
      if (A[idx[j]][idx[j]] < A[idx[i]][idx[i]]) {
        int tmp = idx[i];
        idx[i] = idx[j];
        idx[j] = tmp;
      }
  for (int k = 0; k < 4; ++k) {
    vals[k] = A[idx[k]][idx[k]];
    for (int i = 0; i < 4; ++i) vecs[i + 4 * k] = V[i][idx[k]];
  }
}

int oracle_trace_stride(void) { return ORACLE_TRACE_STRIDE; }

/* OpenMP thread count for the restatement (the CPU-baseline timing uses all cores). */
void oracle_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
}
int oracle_max_threads(void) { return omp_get_max_threads(); }

#define REAL double
#define SUFFIX _f64
#define EXP exp
#define SQRT sqrt
#include "oracle_impl.h"
#undef REAL
#undef SUFFIX
#undef EXP
#undef SQRT

#define REAL float
#define SUFFIX _f32
#define EXP expf
#define SQRT sqrtf
#include "oracle_impl.h"
#undef REAL
#undef SUFFIX
#undef EXP
#undef SQRT
