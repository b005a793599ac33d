// Horn's closed-form absolute orientation (unit-quaternion method), the pose
// update of every registration loop: findRTfromS + eigenvectorOfN,
// src/findRTfromS.cpp:33-159. The reference builds the symmetric 4x4 matrix N
// from the 3x3 cross-covariance S, takes the eigenvector of N's largest
// eigenvalue with LAPACK dsyev_, converts it to R and sets t = Xc - R*Yc.
//
// Here the eigenvector comes from a cyclic Jacobi iteration written for a 4x4
// matrix. It works for T = float (device, one thread per block) and T = double
// (host C ABI). The device path keeps the previous step's eigenbasis V and
// starts each solve from B = V^T N V. Consecutive annealing steps change N
// only slightly, so one or two sweeps reach FP32 round-off. Each solve
// re-orthonormalises V with one Newton-Schulz step. Kernels that need no
// eigenbasis (no adjoint tape) first try a certified shifted inverse
// iteration from the previous quaternion (horn_quaternion_fast), several
// times cheaper, and fall back to the Jacobi solve.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define CESA_HD __host__ __device__ __forceinline__
#else
#define CESA_HD inline
#endif

namespace cesa {

template <typename T>
CESA_HD T t_abs(T x) {
  return x < T(0) ? -x : x;
}
template <typename T>
CESA_HD bool t_finite(T x) {
  return x == x && t_abs(x) <= T(3.0e38);
}
CESA_HD float t_rsqrt(float x) {
#if defined(__CUDA_ARCH__)
  return rsqrtf(x);
#else
  return 1.0f / sqrtf(x);
#endif
}
CESA_HD double t_rsqrt(double x) { return 1.0 / sqrt(x); }
// a / b; the device FP32 path uses the approximate (MUFU) division: Jacobi
// only needs each rotation to be orthogonal (c = rsqrt(1 + t^2), s = t c),
// not the exact angle.
CESA_HD float t_div(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
CESA_HD double t_div(double a, double b) { return a / b; }

template <typename T>
struct HornState {
  T V[4][4];   // eigenbasis carried between solves (warm start)
  T q[4];      // last good quaternion (fallback when N is not finite)
  CESA_HD void reset() {
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) V[i][j] = (i == j) ? T(1) : T(0);
    q[0] = T(1);
    q[1] = q[2] = q[3] = T(0);
  }
};

// One Jacobi rotation of the symmetric B in the (p,q) plane: computes (c, s)
// that zero B[p][q] (Numerical-Recipes convention theta = (bqq-bpp)/(2 bpq)).
template <typename T>
CESA_HD bool jacobi_angle(T bpp, T bqq, T bpq, T tol, T& c, T& s, T& tmax) {
  if (t_abs(bpq) <= tol) {
    c = T(1);
    s = T(0);
    return false;
  }
  const T d = bqq - bpp;
  // t = 2 bpq sgn(d) / (|d| + sqrt(d^2 + 4 bpq^2)), the smaller root.
  const T r2 = d * d + T(4) * bpq * bpq;
  const T r = r2 * t_rsqrt(r2);
  const T den = t_abs(d) + r;
  T t = t_div(T(2) * bpq, den);
  if (d < T(0)) t = -t;
  tmax = t_abs(t) > tmax ? t_abs(t) : tmax;
  c = t_rsqrt(T(1) + t * t);
  s = t * c;
  return true;
}

template <typename T, int P, int Q>
CESA_HD void jacobi_apply(T (&B)[4][4], T (&W)[4][4], T c, T s) {
  // B <- J^T B J with J = I except J[P][P]=J[Q][Q]=c, J[P][Q]=s, J[Q][P]=-s.
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T bkp = B[k][P], bkq = B[k][Q];
    B[k][P] = c * bkp - s * bkq;
    B[k][Q] = s * bkp + c * bkq;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T bpk = B[P][k], bqk = B[Q][k];
    B[P][k] = c * bpk - s * bqk;
    B[Q][k] = s * bpk + c * bqk;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const T wkp = W[k][P], wkq = W[k][Q];
    W[k][P] = c * wkp - s * wkq;
    W[k][Q] = s * wkp + c * wkq;
  }
}

// Two disjoint rotations per round: {(0,1),(2,3)}, {(0,2),(1,3)}, {(0,3),(1,2)}.
template <typename T, int P1, int Q1, int P2, int Q2>
CESA_HD bool jacobi_round(T (&B)[4][4], T (&W)[4][4], T tol, T& tmax) {
  T c1, s1, c2, s2;
  const bool r1 = jacobi_angle<T>(B[P1][P1], B[Q1][Q1], B[P1][Q1], tol, c1, s1, tmax);
  const bool r2 = jacobi_angle<T>(B[P2][P2], B[Q2][Q2], B[P2][Q2], tol, c2, s2, tmax);
  if (r1) jacobi_apply<T, P1, Q1>(B, W, c1, s1);
  if (r2) jacobi_apply<T, P2, Q2>(B, W, c2, s2);
  return r1 || r2;
}

// Horn's N from S in the reference's h_S layout (src/findRTfromS.cpp:38-74).
template <typename T>
CESA_HD void horn_matrix(const T S[9], T (&N)[4][4]) {
  const T Sxx = S[0], Sxy = S[1], Sxz = S[2];
  const T Syx = S[3], Syy = S[4], Syz = S[5];
  const T Szx = S[6], Szy = S[7], Szz = S[8];
  N[0][0] = Sxx + Syy + Szz;
  N[0][1] = N[1][0] = Syz - Szy;
  N[0][2] = N[2][0] = Szx - Sxz;
  N[0][3] = N[3][0] = Sxy - Syx;
  N[1][1] = Sxx - Syy - Szz;
  N[1][2] = N[2][1] = Sxy + Syx;
  N[1][3] = N[3][1] = Szx + Sxz;
  N[2][2] = Syy - Sxx - Szz;
  N[2][3] = N[3][2] = Syz + Szy;
  N[3][3] = Szz - Sxx - Syy;
}

// Quaternion -> rotation (src/findRTfromS.cpp:83-91) and t = Xc - R Yc (:94-96).
template <typename T>
CESA_HD void quat_to_pose(const T q[4], const T Xc[3], const T Yc[3], T R[9], T t[3]) {
  const T q0 = q[0], qx = q[1], qy = q[2], qz = q[3];
  R[0] = q0 * q0 + qx * qx - qy * qy - qz * qz;
  R[1] = T(2) * (qx * qy - q0 * qz);
  R[2] = T(2) * (qx * qz + q0 * qy);
  R[3] = T(2) * (qy * qx + q0 * qz);
  R[4] = q0 * q0 - qx * qx + qy * qy - qz * qz;
  R[5] = T(2) * (qy * qz - q0 * qx);
  R[6] = T(2) * (qz * qx - q0 * qy);
  R[7] = T(2) * (qz * qy + q0 * qx);
  R[8] = q0 * q0 - qx * qx - qy * qy + qz * qz;
  for (int i = 0; i < 3; ++i) t[i] = Xc[i] - (R[3 * i] * Yc[0] + R[3 * i + 1] * Yc[1] + R[3 * i + 2] * Yc[2]);
}

// Top eigenvector of Horn's N for S; warm-started from st.V. Writes q (unit)
// and returns 0, or returns 1 and the fallback st.q when N is not finite.
// gap = (l1 - l2)/|l1|, lmax = l1.
template <typename T>
CESA_HD int horn_quaternion(const T S[9], HornState<T>& st, T q[4], T* gap, T* lmax) {
  T N[4][4];
  horn_matrix<T>(S, N);
  bool finite = true;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) finite = finite && t_finite(N[i][j]);
  if (!finite) {
    for (int i = 0; i < 4; ++i) q[i] = st.q[i];
    if (gap) *gap = T(0);
    if (lmax) *lmax = T(0);
    return 1;
  }
  // Work on register copies (static indices only) of the carried basis.
  T V[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) V[i][j] = st.V[i][j];
  // B = V^T N V
  T NV[4][4], B[4][4], W[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      NV[i][j] = N[i][0] * V[0][j] + N[i][1] * V[1][j] + N[i][2] * V[2][j] + N[i][3] * V[3][j];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      B[i][j] = V[0][i] * NV[0][j] + V[1][i] * NV[1][j] + V[2][i] * NV[2][j] + V[3][i] * NV[3][j];
      W[i][j] = (i == j) ? T(1) : T(0);
    }
  // symmetrise (round-off in the two products)
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = i + 1; j < 4; ++j) {
      const T m = T(0.5) * (B[i][j] + B[j][i]);
      B[i][j] = B[j][i] = m;
    }
  // rotations stop once the off-diagonal entries are at round-off level
  T scale = T(0);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) scale = t_abs(N[i][j]) > scale ? t_abs(N[i][j]) : scale;
  const T eps = sizeof(T) == 4 ? T(1.2e-7) : T(2.3e-16);
  const T tol = T(4) * eps * scale + T(1e-37);
  // A sweep whose rotations all have |tan| < sqrt(eps) leaves off-diagonal
  // entries of order tan^2 (relative): the next sweep would change nothing
  // above round-off, so it is not run.
  const T tquad = sizeof(T) == 4 ? T(3.4e-4) : T(1.5e-8);
  for (int sweep = 0; sweep < 16; ++sweep) {
    T tmax = T(0);
    bool rot = jacobi_round<T, 0, 1, 2, 3>(B, W, tol, tmax);
    rot = jacobi_round<T, 0, 2, 1, 3>(B, W, tol, tmax) || rot;
    rot = jacobi_round<T, 0, 3, 1, 2>(B, W, tol, tmax) || rot;
    if (!rot || tmax < tquad) break;
  }
  // V <- V W, then one Newton-Schulz step V <- V (3I - V^T V)/2
  T V2[4][4], G[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      V2[i][j] = V[i][0] * W[0][j] + V[i][1] * W[1][j] + V[i][2] * W[2][j] + V[i][3] * W[3][j];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      G[i][j] = (i == j ? T(1.5) : T(0)) -
                T(0.5) * (V2[0][i] * V2[0][j] + V2[1][i] * V2[1][j] + V2[2][i] * V2[2][j] +
                          V2[3][i] * V2[3][j]);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      V[i][j] = V2[i][0] * G[0][j] + V2[i][1] * G[1][j] + V2[i][2] * G[2][j] + V2[i][3] * G[3][j];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) st.V[i][j] = V[i][j];
  // largest eigenvalue; its column selected without dynamic indexing
  T l1 = B[0][0], l2 = T(-3.0e38);
  int imax = 0;
#pragma unroll
  for (int i = 1; i < 4; ++i)
    if (B[i][i] > l1) {
      l1 = B[i][i];
      imax = i;
    }
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (i != imax && B[i][i] > l2) l2 = B[i][i];
  T qq[4];
  T n2 = T(0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    qq[i] = imax == 0 ? V[i][0] : imax == 1 ? V[i][1] : imax == 2 ? V[i][2] : V[i][3];
    n2 += qq[i] * qq[i];
  }
  const T inv = t_rsqrt(n2);
  bool ok = t_finite(inv);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    qq[i] *= inv;
    ok = ok && t_finite(qq[i]);
  }
  if (!ok) {
    for (int i = 0; i < 4; ++i) q[i] = st.q[i];
    st.reset();
    if (gap) *gap = T(0);
    if (lmax) *lmax = T(0);
    return 1;
  }
  for (int i = 0; i < 4; ++i) q[i] = st.q[i] = qq[i];
  if (gap) *gap = t_div(l1 - l2, t_abs(l1) > T(1e-30) ? t_abs(l1) : T(1e-30));
  if (lmax) *lmax = l1;
  return 0;
}

// Cholesky factor L (lower) of a symmetric 4x4 A, with the reciprocals of its
// diagonal in rd. False when a pivot is not positive and finite, i.e. when A
// is not (numerically) positive definite.
template <typename T>
CESA_HD bool chol4(const T (&A)[4][4], T (&L)[4][4], T (&rd)[4]) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    T d = A[j][j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= L[j][k] * L[j][k];
    if (!(d > T(0)) || !t_finite(d)) return false;
    const T r = t_rsqrt(d);
    rd[j] = r;
    L[j][j] = d * r;
#pragma unroll
    for (int i = j + 1; i < 4; ++i) {
      T v = A[i][j];
#pragma unroll
      for (int k = 0; k < j; ++k) v -= L[i][k] * L[j][k];
      L[i][j] = v * r;
    }
  }
  return true;
}

// x = (L L^T)^-1 b, normalised to unit length.
template <typename T>
CESA_HD void chol4_solve_unit(const T (&L)[4][4], const T (&rd)[4], const T (&b)[4], T (&x)[4]) {
  T y[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    T v = b[i];
#pragma unroll
    for (int k = 0; k < i; ++k) v -= L[i][k] * y[k];
    y[i] = v * rd[i];
  }
#pragma unroll
  for (int i = 3; i >= 0; --i) {
    T v = y[i];
#pragma unroll
    for (int k = i + 1; k < 4; ++k) v -= L[k][i] * x[k];
    x[i] = v * rd[i];
  }
  const T inv = t_rsqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + x[3] * x[3]);
#pragma unroll
  for (int i = 0; i < 4; ++i) x[i] *= inv;
}

// Shifted A = sigma I - N - c v v^T (c < 0 deflates v out of N's spectrum).
template <typename T>
CESA_HD void shifted4(const T (&N)[4][4], T sigma, T c, const T (&v)[4], T (&A)[4][4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) A[i][j] = (i == j ? sigma : T(0)) - N[i][j] - c * v[i] * v[j];
}

// Top eigenvector of the symmetric N by shifted inverse iteration from q0, a
// unit vector near it (the previous pose update's quaternion). The shift
// lambda(q0) + 2e-5 max|N| is tried first (a warm q0 is close enough that it
// lies above the top eigenvalue); where that matrix does not factor, one step
// with lambda(q0) + 1e-3 max|N| comes first. A shift that factors (sigma I - N
// positive definite) lies above the largest eigenvalue, so the iteration
// converges to its eigenvector: one solve, a second when the residual is not
// yet at round-off. The result is certified, else refused (false): with r the
// residual N v - lambda v, the Davis-Kahan bound sin(angle to the true
// eigenvector) <= |r| / gap holds, and the gap is certified by factoring
// (lambda - g) I - (N - (lambda + max|N|) v v^T), N with v deflated out of its
// spectrum: positive definite exactly when every other eigenvalue is below
// lambda - g. g is set so that the bound is 4e-6 (and at
// least 2% of max|N|). Typically two 4x4 Cholesky factorisations and one
// solve.
template <typename T>
CESA_HD bool horn_top_inverse(const T (&N)[4][4], const T (&q0)[4], T (&q)[4], T* lmax) {
  // max |N_ij| as a tree (the same value as a running maximum, fewer dependent steps)
  T mx[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) mx[k] = t_abs(N[k / 4][k % 4]);
#pragma unroll
  for (int w = 8; w >= 1; w /= 2)
#pragma unroll
    for (int k = 0; k < w; ++k) mx[k] = mx[k + w] > mx[k] ? mx[k + w] : mx[k];
  const T scale = mx[0];
  if (!(scale > T(1e-30)) || !t_finite(scale)) return false;
  T v[4], x[4], Nv[4], A[4][4], L[4][4], rd[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = q0[i];
#pragma unroll
  for (int i = 0; i < 4; ++i) Nv[i] = N[i][0] * v[0] + N[i][1] * v[1] + N[i][2] * v[2] + N[i][3] * v[3];
  T lam = v[0] * Nv[0] + v[1] * Nv[1] + v[2] * Nv[2] + v[3] * Nv[3];
  shifted4<T>(N, lam + T(2e-5) * scale, T(0), v, A);
  if (!chol4<T>(A, L, rd)) {
    shifted4<T>(N, lam + T(1e-3) * scale, T(0), v, A);
    if (!chol4<T>(A, L, rd)) return false;
    chol4_solve_unit<T>(L, rd, v, x);
#pragma unroll
    for (int i = 0; i < 4; ++i) Nv[i] = N[i][0] * x[0] + N[i][1] * x[1] + N[i][2] * x[2] + N[i][3] * x[3];
    lam = x[0] * Nv[0] + x[1] * Nv[1] + x[2] * Nv[2] + x[3] * Nv[3];
    shifted4<T>(N, lam + T(2e-5) * scale, T(0), x, A);
    if (!chol4<T>(A, L, rd)) return false;
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = x[i];
  }
  T rn = T(0);
  for (int it = 0; it < 2; ++it) {
    chol4_solve_unit<T>(L, rd, v, x);
    // residual and Rayleigh quotient of x
#pragma unroll
    for (int i = 0; i < 4; ++i) Nv[i] = N[i][0] * x[0] + N[i][1] * x[1] + N[i][2] * x[2] + N[i][3] * x[3];
    lam = x[0] * Nv[0] + x[1] * Nv[1] + x[2] * Nv[2] + x[3] * Nv[3];
    T r2 = T(0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const T ri = Nv[i] - lam * x[i];
      r2 += ri * ri;
    }
    rn = r2 * t_rsqrt(r2 > T(0) ? r2 : T(1e-37));
    if (rn <= T(4e-6) * T(0.02) * scale) break;  // already within the bound at the smallest gap
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = x[i];
  }
  T g = rn / T(4e-6);
  if (g < T(0.02) * scale) g = T(0.02) * scale;
  shifted4<T>(N, lam - g, -(lam + scale), x, A);
  if (!chol4<T>(A, L, rd) || !t_finite(lam)) return false;
  // the sign that continues the previous quaternion
  const T s = x[0] * q0[0] + x[1] * q0[1] + x[2] * q0[2] + x[3] * q0[3] < T(0) ? T(-1) : T(1);
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i] = s * x[i];
  if (lmax) *lmax = lam;
  return true;
}

// Horn's top eigenvector for the plain forward kernels: the certified inverse
// iteration from the previous quaternion (st.q), else the warm-started Jacobi
// of horn_quaternion (whose basis st.V it then refreshes). gap is reported
// only by the Jacobi path; the inverse iteration writes -1 (its certificate
// is gap >= 2% of max|N|). Returns 1 when N is not finite (st.q kept).
template <typename T>
CESA_HD int horn_quaternion_fast(const T S[9], HornState<T>& st, T q[4], T* gap, T* lmax) {
  T N[4][4];
  horn_matrix<T>(S, N);
  bool finite = true;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) finite = finite && t_finite(N[i][j]);
  if (finite) {
    T q0[4], qq[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) q0[i] = st.q[i];
    if (horn_top_inverse<T>(N, q0, qq, lmax)) {
#pragma unroll
      for (int i = 0; i < 4; ++i) q[i] = st.q[i] = qq[i];
      if (gap) *gap = T(-1);
      return 0;
    }
  }
  return horn_quaternion<T>(S, st, q, gap, lmax);
}

// Adjoint of the pose update (R, t) = (R(q), Xc - R(q) Yc) with q the top
// eigenvector of Horn's N(S) (horn_matrix, quat_to_pose): from dL/dR (9,
// row-major) and dL/dt of the output, dL/dS (h_S layout), dL/dXc and dL/dYc.
// V: the eigenbasis of N(S) (columns; as left by horn_quaternion), q the
// quaternion used. Eigenvalues are Rayleigh quotients; the column closest to q
// is the top one; dq = sum over the other eigenvectors of v_j (v_j^T dN q) /
// (l_top - l_j).
template <typename T>
CESA_HD void horn_pose_adjoint(const T S[9], const T Xc[3], const T Yc[3], const T q[4], const T (&V)[4][4],
                               const T gRo[9], const T gto[3], T gS[9], T gXc[3], T gYc[3]) {
  T R[9], tdummy[3];
  quat_to_pose<T>(q, Xc, Yc, R, tdummy);
  // t = Xc - R Yc
  T gR[9];
  for (int i = 0; i < 3; ++i) gXc[i] = gto[i];
  for (int j = 0; j < 3; ++j) gYc[j] = -(R[j] * gto[0] + R[3 + j] * gto[1] + R[6 + j] * gto[2]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) gR[3 * i + j] = gRo[3 * i + j] - gto[i] * Yc[j];
  // R(q): dR_k / dq_a = 2 dR[k][a]
  const T q0 = q[0], qx = q[1], qy = q[2], qz = q[3];
  const T dR[9][4] = {{q0, qx, -qy, -qz}, {-qz, qy, qx, -q0}, {qy, qz, q0, qx},
                      {qz, qy, qx, q0},   {q0, -qx, qy, -qz}, {-qx, -q0, qz, qy},
                      {-qy, qz, -q0, qx}, {qx, q0, qz, qy},   {q0, -qx, -qy, qz}};
  T gq[4] = {T(0), T(0), T(0), T(0)};
  for (int k = 0; k < 9; ++k)
    for (int a = 0; a < 4; ++a) gq[a] += T(2) * gR[k] * dR[k][a];
  T N[4][4];
  horn_matrix<T>(S, N);
  T lam[4];
  int top = 0;
  T best = T(-1);
  for (int j = 0; j < 4; ++j) {
    T nv[4], vv = T(0), vq = T(0);
    for (int i = 0; i < 4; ++i) nv[i] = N[i][0] * V[0][j] + N[i][1] * V[1][j] + N[i][2] * V[2][j] + N[i][3] * V[3][j];
    lam[j] = T(0);
    for (int i = 0; i < 4; ++i) {
      lam[j] += V[i][j] * nv[i];
      vv += V[i][j] * V[i][j];
      vq += V[i][j] * q[i];
    }
    lam[j] = t_div(lam[j], vv);
    const T a = t_abs(vq) * t_rsqrt(vv);
    if (a > best) {
      best = a;
      top = j;
    }
  }
  T G[4][4];
  for (int i = 0; i < 4; ++i)
    for (int k = 0; k < 4; ++k) G[i][k] = T(0);
  for (int j = 0; j < 4; ++j) {
    if (j == top) continue;
    T vv = T(0), vg = T(0);
    for (int i = 0; i < 4; ++i) {
      vv += V[i][j] * V[i][j];
      vg += V[i][j] * gq[i];
    }
    const T c = t_div(vg, vv * (lam[top] - lam[j]));
    for (int i = 0; i < 4; ++i)
      for (int k = 0; k < 4; ++k) G[i][k] += c * V[i][j] * q[k];
  }
  // N(S) is linear in S (horn_matrix); its adjoint
  const T a01 = G[0][1] + G[1][0], a02 = G[0][2] + G[2][0], a03 = G[0][3] + G[3][0];
  const T a12 = G[1][2] + G[2][1], a13 = G[1][3] + G[3][1], a23 = G[2][3] + G[3][2];
  gS[0] = G[0][0] + G[1][1] - G[2][2] - G[3][3];  // Sxx
  gS[4] = G[0][0] - G[1][1] + G[2][2] - G[3][3];  // Syy
  gS[8] = G[0][0] - G[1][1] - G[2][2] + G[3][3];  // Szz
  gS[5] = a01 + a23;                              // Syz
  gS[7] = -a01 + a23;                             // Szy
  gS[6] = a02 + a13;                              // Szx
  gS[2] = -a02 + a13;                             // Sxz
  gS[1] = a03 + a12;                              // Sxy
  gS[3] = -a03 + a12;                             // Syx
}

}  // namespace cesa
