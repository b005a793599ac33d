/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- the product never links or calls this.
 *
 * Precision-generic body of the CPU restatement of the reference's two soft
 * registration loops. cesa_oracle.c includes this file twice:
 *   REAL = double  -> *_f64, the parity oracle;
 *   REAL = float   -> *_f32, a port that keeps the reference's FP32
 *                     arithmetic, used as the timed CPU baseline.
 * The annealing schedules (sigma_p2 and T) are stepped in FP32 in both, as the
 * reference's loop variables are floats (src/emicp.cu:262,668;
 * src/softassign.cu:277,820).
 *
 * Trace record per pose update (ORACLE_TRACE_STRIDE doubles):
 *   [0] step  [1] sigma_p2 or T  [2] sum(lambda) or sumM  [3..5] Xc  [6..8] Yc
 *   [9..17] S (h_S layout: S[i+3j] = sum X-side_i * Y-side_j)
 *   [18..26] R row-major  [27..29] t  [30] relative eigen-gap of Horn's N
 *   [31] largest eigenvalue of N
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUFFIX)

/*
 * EM-ICP, one sigma step: E-step (updateA, row sums + outlier term,
 * normalizeRowsOfA) and the weighted moments (lambda, X', Xc, Yc, S).
 * Follows src/emicp_cpu.cpp:311-495 (== src/emicp.cu:453-624).
 * Rows are Y points (rowsA = M), columns are X points (colsA = N).
 * Outputs per row (optional): C[r] (row sum incl. outlier term), lam[r],
 * U[r*3+i] = lam_r * X'_r,i.  Returns sum(lambda) and fills Xc, Yc, S.
 */
static double FN(emicp_moments)(const float* X, int N, const float* Y, int M, const REAL R[9],
                                const REAL t[3], float sigma_p2, float d_02, REAL* C_out,
                                REAL* lam_out, REAL* U_out, REAL Xc[3], REAL Yc[3], REAL S[9]) {
  const float* Xx = X;
  const float* Xy = X + N;
  const float* Xz = X + 2 * N;
  const float* Yx = Y;
  const float* Yy = Y + M;
  const float* Yz = Y + 2 * M;
  /* src/emicp_cpu.cpp:356 -- expf(-d_02/sigma_p2) in FP32 on the host */
  const REAL outlier = EXP(-(REAL)d_02 / (REAL)sigma_p2);
  const REAL s2 = (REAL)sigma_p2;
  const REAL thresh = (REAL)10e-7f; /* src/emicp_cpu.cpp:121, i.e. 1e-6 */
  REAL* lam = (REAL*)malloc(sizeof(REAL) * (size_t)(M > 0 ? M : 1));
  REAL* U = (REAL*)malloc(sizeof(REAL) * 3 * (size_t)(M > 0 ? M : 1));

#pragma omp parallel
  {
    REAL* A = (REAL*)malloc(sizeof(REAL) * (size_t)(N > 0 ? N : 1));
#pragma omp for schedule(static)
    for (int r = 0; r < M; ++r) {
      /* updateA, src/emicp_cpu.cpp:92-106: A(r,c) = exp(-|x_c - (R y_r + t)|^2 / sigma_p2) */
      REAL sumA = 0;
      for (int c = 0; c < N; ++c) {
        REAL dx = (REAL)Xx[c] - (R[0] * Yx[r] + R[1] * Yy[r] + R[2] * Yz[r] + t[0]);
        REAL dy = (REAL)Xy[c] - (R[3] * Yx[r] + R[4] * Yy[r] + R[5] * Yz[r] + t[1]);
        REAL dz = (REAL)Xz[c] - (R[6] * Yx[r] + R[7] * Yy[r] + R[8] * Yz[r] + t[2]);
        REAL d2 = dx * dx + dy * dy + dz * dz;
        A[c] = EXP(-d2 / s2);
        sumA += A[c];
      }
      /* row sum plus outlier term, src/emicp_cpu.cpp:342-358 */
      REAL Cr = sumA + outlier;
      REAL l = 0, ux = 0, uy = 0, uz = 0;
      if (Cr > thresh) {
        /* normalizeRowsOfA, src/emicp_cpu.cpp:121-123: A <- sqrt(A / C) */
        for (int c = 0; c < N; ++c) {
          REAL a = SQRT(A[c] / Cr);
          l += a;
          ux += a * Xx[c];
          uy += a * Xy[c];
          uz += a * Xz[c];
        }
      } else {
        /* src/emicp_cpu.cpp:125: A <- 1/colsA */
        REAL a = (REAL)1 / (REAL)N;
        for (int c = 0; c < N; ++c) {
          l += a;
          ux += a * Xx[c];
          uy += a * Xy[c];
          uz += a * Xz[c];
        }
      }
      lam[r] = l;
      U[3 * r + 0] = ux;
      U[3 * r + 1] = uy;
      U[3 * r + 2] = uz;
      if (C_out) C_out[r] = Cr;
    }
    free(A);
  }

  /* sasum, src/emicp_cpu.cpp:391 */
  REAL sumLam = 0;
  for (int r = 0; r < M; ++r) sumLam += (lam[r] < 0 ? -lam[r] : lam[r]);
  /* weighted centres: Xc = X'^T lambda / sum, Yc = Y^T lambda / sum (src/emicp_cpu.cpp:435-460).
   * lam_r * X'_r = U_r; the division X' = U/lam (src/emicp_cpu.cpp:419) is never
   * formed, so a row with lam_r == 0 contributes 0 instead of 0/0. */
  REAL xc[3] = {0, 0, 0}, yc[3] = {0, 0, 0};
  for (int r = 0; r < M; ++r) {
    for (int i = 0; i < 3; ++i) xc[i] += U[3 * r + i];
    yc[0] += lam[r] * Yx[r];
    yc[1] += lam[r] * Yy[r];
    yc[2] += lam[r] * Yz[r];
  }
  for (int i = 0; i < 3; ++i) {
    Xc[i] = xc[i] / sumLam;
    Yc[i] = yc[i] / sumLam;
  }
  /* S = (lam .* (X' - Xc))^T (Y - Yc), src/emicp_cpu.cpp:469-495 */
  for (int k = 0; k < 9; ++k) S[k] = 0;
  for (int r = 0; r < M; ++r) {
    REAL xd[3], yd[3];
    for (int i = 0; i < 3; ++i) xd[i] = U[3 * r + i] - lam[r] * Xc[i];
    yd[0] = Yx[r] - Yc[0];
    yd[1] = Yy[r] - Yc[1];
    yd[2] = Yz[r] - Yc[2];
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) S[i + 3 * j] += xd[i] * yd[j];
  }
  if (lam_out) memcpy(lam_out, lam, sizeof(REAL) * (size_t)M);
  if (U_out) memcpy(U_out, U, sizeof(REAL) * 3 * (size_t)M);
  free(lam);
  free(U);
  return (double)sumLam;
}

static void FN(trace_put)(double* rec, int step, double sched, double sum, const REAL Xc[3],
                          const REAL Yc[3], const REAL S[9], const REAL R[9], const REAL t[3],
                          double gap, double lmax) {
  rec[0] = step;
  rec[1] = sched;
  rec[2] = sum;
  for (int i = 0; i < 3; ++i) {
    rec[3 + i] = Xc[i];
    rec[6 + i] = Yc[i];
    rec[27 + i] = t[i];
  }
  for (int i = 0; i < 9; ++i) {
    rec[9 + i] = S[i];
    rec[18 + i] = R[i];
  }
  rec[30] = gap;
  rec[31] = lmax;
}

/* Horn's pose from (Xc, Yc, S) in REAL precision; the eigen-solve is always FP64. */
static void FN(pose_update)(const REAL Xc[3], const REAL Yc[3], const REAL S[9], REAL R[9],
                            REAL t[3], double q_prev[4], double* gap, double* lmax) {
  double xc[3], yc[3], s[9], r[9], tt[3];
  for (int i = 0; i < 3; ++i) {
    xc[i] = Xc[i];
    yc[i] = Yc[i];
  }
  for (int i = 0; i < 9; ++i) s[i] = S[i];
  oracle_find_rt_from_s(xc, yc, s, r, tt, q_prev, gap, lmax);
  for (int i = 0; i < 9; ++i) R[i] = (REAL)r[i];
  /* t = Xc - R Yc with the rounded R, as src/findRTfromS.cpp:94-96 */
  for (int i = 0; i < 3; ++i) t[i] = Xc[i] - (R[3 * i] * Yc[0] + R[3 * i + 1] * Yc[1] + R[3 * i + 2] * Yc[2]);
}

/*
 * Full annealed EM-ICP, src/emicp_cpu.cpp:303-528.
 * R (row-major) and t are the initial pose on entry, the estimate on exit.
 * Returns the number of sigma steps.
 */
int FN(oracle_emicp)(const float* X, int N, const float* Y, int M, REAL R[9], REAL t[3],
                     float sigma_p2, float sigma_inf, float sigma_factor, float d_02,
                     double* trace, int trace_cap) {
  if (N <= 0 || M <= 0) return -1;
  double q_prev[4] = {1, 0, 0, 0};
  int step = 0;
  while (sigma_p2 > sigma_inf) {
    REAL Xc[3], Yc[3], S[9];
    double sumLam =
        FN(emicp_moments)(X, N, Y, M, R, t, sigma_p2, d_02, NULL, NULL, NULL, Xc, Yc, S);
    double gap = 0, lmax = 0;
    FN(pose_update)(Xc, Yc, S, R, t, q_prev, &gap, &lmax);
    if (trace && step < trace_cap)
      FN(trace_put)(trace + (size_t)ORACLE_TRACE_STRIDE * step, step, sigma_p2, sumLam, Xc, Yc, S,
                    R, t, gap, lmax);
    ++step;
    sigma_p2 *= sigma_factor; /* FP32, src/emicp_cpu.cpp:527 */
  }
  return step;
}

/* One E-step with per-row outputs, for unit-level parity of the fused kernel. */
double FN(oracle_emicp_step)(const float* X, int N, const float* Y, int M, const REAL R[9],
                             const REAL t[3], float sigma_p2, float d_02, REAL* C_out,
                             REAL* lam_out, REAL* U_out, REAL Xc[3], REAL Yc[3], REAL S[9]) {
  return FN(emicp_moments)(X, N, Y, M, R, t, sigma_p2, d_02, C_out, lam_out, U_out, Xc, Yc, S);
}

/*
 * Softassign, one inner iteration at temperature T (src/softassign.cu:494-798).
 * Mtx is a caller-provided N x M scratch (row-major, rows = X points).
 * s[N], u[M] are the persistent slack column / row (in/out).
 * Outputs: rs[N] (last row sums incl. slack), cs[M] (last column sums incl.
 * slack, taken before the last column normalisation), w[N] (row sums of the
 * final M, no slack); returns sumM and fills Xc, Yc, S.
 */
static double FN(softassign_inner)(const float* X, int N, const float* Y, int M, const REAL R[9],
                                   const REAL t[3], float T_cur, float alpha, int I1, REAL* Mtx,
                                   REAL* s, REAL* u, REAL* rs, REAL* cs, REAL* w, REAL Xc[3],
                                   REAL Yc[3], REAL S[9]) {
  const float* Xx = X;
  const float* Xy = X + N;
  const float* Xz = X + 2 * N;
  const float* Yx = Y;
  const float* Yy = Y + M;
  const float* Yz = Y + 2 * M;
  const REAL T = (REAL)T_cur;
  const REAL sqT = SQRT(T);
  /* updateM, src/softassign.cu:106-135: M = exp(-(|x_r - (R y_c + t)|^2 - alpha)/T)/sqrt(T) */
#pragma omp parallel for schedule(static)
  for (int r = 0; r < N; ++r) {
    REAL* row = Mtx + (size_t)r * M;
    for (int c = 0; c < M; ++c) {
      REAL dx = (REAL)Xx[r] - (R[0] * Yx[c] + R[1] * Yy[c] + R[2] * Yz[c] + t[0]);
      REAL dy = (REAL)Xy[r] - (R[3] * Yx[c] + R[4] * Yy[c] + R[5] * Yz[c] + t[1]);
      REAL dz = (REAL)Xz[r] - (R[6] * Yx[c] + R[7] * Yy[c] + R[8] * Yz[c] + t[2]);
      REAL d2 = dx * dx + dy * dy + dz * dz;
      d2 -= (REAL)alpha;
      row[c] = EXP(-d2 / T) / sqT;
    }
  }
  /* Sinkhorn with slack, src/softassign.cu:522-599 */
  for (int k = 0; k < I1; ++k) {
#pragma omp parallel for schedule(static)
    for (int r = 0; r < N; ++r) {
      REAL* row = Mtx + (size_t)r * M;
      REAL sum = 0;
      for (int c = 0; c < M; ++c) sum += row[c];
      sum += s[r];
      rs[r] = sum;
      for (int c = 0; c < M; ++c) row[c] /= sum;
      s[r] /= sum;
    }
    for (int c = 0; c < M; ++c) cs[c] = 0;
#pragma omp parallel
    {
      REAL* part = (REAL*)calloc((size_t)M, sizeof(REAL));
#pragma omp for schedule(static)
      for (int r = 0; r < N; ++r) {
        const REAL* row = Mtx + (size_t)r * M;
        for (int c = 0; c < M; ++c) part[c] += row[c];
      }
#pragma omp critical
      for (int c = 0; c < M; ++c) cs[c] += part[c];
      free(part);
    }
    for (int c = 0; c < M; ++c) cs[c] += u[c];
#pragma omp parallel for schedule(static)
    for (int r = 0; r < N; ++r) {
      REAL* row = Mtx + (size_t)r * M;
      for (int c = 0; c < M; ++c) row[c] /= cs[c];
    }
    for (int c = 0; c < M; ++c) u[c] /= cs[c];
  }
  /* w = M 1 (no slack), sumM = sum |w| -- src/softassign.cu:626-639 */
#pragma omp parallel for schedule(static)
  for (int r = 0; r < N; ++r) {
    const REAL* row = Mtx + (size_t)r * M;
    REAL sum = 0;
    for (int c = 0; c < M; ++c) sum += row[c];
    w[r] = sum;
  }
  REAL sumM = 0;
  for (int r = 0; r < N; ++r) sumM += (w[r] < 0 ? -w[r] : w[r]);
  /* weighted then centred X and Y, src/softassign.cu:653-735.
   * Y is weighted by the last column sums cs (stale, slack included). */
  REAL xc[3] = {0, 0, 0}, yc[3] = {0, 0, 0};
  for (int r = 0; r < N; ++r) {
    xc[0] += w[r] * Xx[r];
    xc[1] += w[r] * Xy[r];
    xc[2] += w[r] * Xz[r];
  }
  for (int c = 0; c < M; ++c) {
    yc[0] += cs[c] * Yx[c];
    yc[1] += cs[c] * Yy[c];
    yc[2] += cs[c] * Yz[c];
  }
  for (int i = 0; i < 3; ++i) {
    Xc[i] = xc[i] / sumM;
    Yc[i] = yc[i] / sumM;
  }
  REAL* Yw = (REAL*)malloc(sizeof(REAL) * 3 * (size_t)M);
  for (int c = 0; c < M; ++c) {
    Yw[3 * c + 0] = cs[c] * Yx[c] - Yc[0];
    Yw[3 * c + 1] = cs[c] * Yy[c] - Yc[1];
    Yw[3 * c + 2] = cs[c] * Yz[c] - Yc[2];
  }
  /* D = M Yw (N x 3), S = Xw^T D -- src/softassign.cu:761-772 */
  REAL Sacc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma omp parallel
  {
    REAL Sl[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma omp for schedule(static)
    for (int r = 0; r < N; ++r) {
      const REAL* row = Mtx + (size_t)r * M;
      REAL D[3] = {0, 0, 0};
      for (int c = 0; c < M; ++c) {
        D[0] += row[c] * Yw[3 * c + 0];
        D[1] += row[c] * Yw[3 * c + 1];
        D[2] += row[c] * Yw[3 * c + 2];
      }
      REAL xw[3] = {w[r] * Xx[r] - Xc[0], w[r] * Xy[r] - Xc[1], w[r] * Xz[r] - Xc[2]};
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) Sl[i + 3 * j] += xw[i] * D[j];
    }
#pragma omp critical
    for (int k = 0; k < 9; ++k) Sacc[k] += Sl[k];
  }
  for (int k = 0; k < 9; ++k) S[k] = Sacc[k];
  free(Yw);
  return (double)sumM;
}

/*
 * Full annealed Softassign, src/softassign.cu:486-822.
 * Returns the number of pose updates (JMAX * I0), or -1 on bad arguments.
 */
int FN(oracle_softassign)(const float* X, int N, const float* Y, int M, REAL R[9], REAL t[3],
                          int JMAX, int I0, int I1, float alpha, float T_0, float TFACTOR,
                          float moutlier, double* trace, int trace_cap) {
  if (N <= 0 || M <= 0 || I1 <= 0) return -1;
  REAL* Mtx = (REAL*)malloc(sizeof(REAL) * (size_t)N * (size_t)M);
  REAL* s = (REAL*)malloc(sizeof(REAL) * (size_t)N);
  REAL* u = (REAL*)malloc(sizeof(REAL) * (size_t)M);
  REAL* rs = (REAL*)malloc(sizeof(REAL) * (size_t)N);
  REAL* cs = (REAL*)malloc(sizeof(REAL) * (size_t)M);
  REAL* w = (REAL*)malloc(sizeof(REAL) * (size_t)N);
  if (!Mtx || !s || !u || !rs || !cs || !w) {
    free(Mtx); free(s); free(u); free(rs); free(cs); free(w);
    return -2;
  }
  /* slack initialised once, src/softassign.cu:385-390 */
  for (int r = 0; r < N; ++r) s[r] = (REAL)moutlier;
  for (int c = 0; c < M; ++c) u[c] = (REAL)moutlier;
  double q_prev[4] = {1, 0, 0, 0};
  float T_cur = T_0;
  int step = 0;
  for (int Titer = 1; Titer <= JMAX; ++Titer) {
    for (int iter0 = 0; iter0 < I0; ++iter0) {
      REAL Xc[3], Yc[3], S[9];
      double sumM = FN(softassign_inner)(X, N, Y, M, R, t, T_cur, alpha, I1, Mtx, s, u, rs, cs,
                                         w, Xc, Yc, S);
      double gap = 0, lmax = 0;
      FN(pose_update)(Xc, Yc, S, R, t, q_prev, &gap, &lmax);
      if (trace && step < trace_cap)
        FN(trace_put)(trace + (size_t)ORACLE_TRACE_STRIDE * step, step, T_cur, sumM, Xc, Yc, S, R,
                      t, gap, lmax);
      ++step;
    }
    T_cur = T_cur * TFACTOR; /* FP32, src/softassign.cu:820 */
  }
  free(Mtx); free(s); free(u); free(rs); free(cs); free(w);
  return step;
}

/*
 * One Softassign inner iteration with all intermediate vectors exposed
 * (unit-level parity of the Sinkhorn sweeps). s and u are in/out.
 */
double FN(oracle_softassign_step)(const float* X, int N, const float* Y, int M, const REAL R[9],
                                  const REAL t[3], float T_cur, float alpha, int I1, REAL* s,
                                  REAL* u, REAL* rs, REAL* cs, REAL* w, REAL Xc[3], REAL Yc[3],
                                  REAL S[9]) {
  if (N <= 0 || M <= 0 || I1 <= 0) return -1.0;
  REAL* Mtx = (REAL*)malloc(sizeof(REAL) * (size_t)N * (size_t)M);
  if (!Mtx) return -2.0;
  double r = FN(softassign_inner)(X, N, Y, M, R, t, T_cur, alpha, I1, Mtx, s, u, rs, cs, w, Xc,
                                  Yc, S);
  free(Mtx);
  return r;
}

/*
 * ICP, src/icp.cpp:122-290: Yc = mean(Y) once; per iteration every y is moved
 * by the current pose and matched to its nearest X point; Xc = mean of the
 * matches, S = sum (x_nn - Xc)(y - Yc)^T (h_S layout, src/icp.cpp:251-262),
 * pose = findRTfromS(Xc, Yc, S); maxIteration iterations, no convergence test.
 * The reference searches with FLANN's randomised kd-trees and default search
 * checks (src/icp.cpp:170-175,211-216), which is approximate; this
 * restatement searches exhaustively and keeps the first of equal distances
 * (lowest X index). nn_out (optional, M): the matches of the last iteration.
 * Trace [2] holds the sum of squared match distances of the iteration.
 */
int FN(oracle_icp)(const float* X, int N, const float* Y, int M, REAL R[9], REAL t[3], int maxIteration,
                   int* nn_out, double* trace, int trace_cap) {
  if (N <= 0 || M <= 0 || maxIteration < 0) return -1;
  const float* Xx = X;
  const float* Xy = X + N;
  const float* Xz = X + 2 * N;
  const float* Yx = Y;
  const float* Yy = Y + M;
  const float* Yz = Y + 2 * M;
  int* nn = (int*)malloc(sizeof(int) * (size_t)M);
  REAL* d2min = (REAL*)malloc(sizeof(REAL) * (size_t)M);
  if (!nn || !d2min) {
    free(nn);
    free(d2min);
    return -2;
  }
  /* findCenter(Y), src/icp.cpp:88-100 */
  REAL Yc[3] = {0, 0, 0};
  for (int i = 0; i < M; ++i) {
    Yc[0] += Yx[i];
    Yc[1] += Yy[i];
    Yc[2] += Yz[i];
  }
  for (int k = 0; k < 3; ++k) Yc[k] /= (REAL)M;
  double q_prev[4] = {1, 0, 0, 0};
  for (int iter = 0; iter < maxIteration; ++iter) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < M; ++i) {
      const REAL zx = R[0] * Yx[i] + R[1] * Yy[i] + R[2] * Yz[i] + t[0];
      const REAL zy = R[3] * Yx[i] + R[4] * Yy[i] + R[5] * Yz[i] + t[1];
      const REAL zz = R[6] * Yx[i] + R[7] * Yy[i] + R[8] * Yz[i] + t[2];
      REAL best = 0;
      int bi = -1;
      for (int c = 0; c < N; ++c) {
        const REAL dx = (REAL)Xx[c] - zx, dy = (REAL)Xy[c] - zy, dz = (REAL)Xz[c] - zz;
        const REAL d2 = dx * dx + dy * dy + dz * dz;
        if (bi < 0 || d2 < best) {
          best = d2;
          bi = c;
        }
      }
      nn[i] = bi;
      d2min[i] = best;
    }
    REAL Xc[3] = {0, 0, 0}, S[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double cost = 0;
    for (int i = 0; i < M; ++i) {
      Xc[0] += Xx[nn[i]];
      Xc[1] += Xy[nn[i]];
      Xc[2] += Xz[nn[i]];
      cost += (double)d2min[i];
    }
    for (int k = 0; k < 3; ++k) Xc[k] /= (REAL)M;
    for (int i = 0; i < M; ++i) {
      const REAL xw[3] = {Xx[nn[i]] - Xc[0], Xy[nn[i]] - Xc[1], Xz[nn[i]] - Xc[2]};
      const REAL yw[3] = {Yx[i] - Yc[0], Yy[i] - Yc[1], Yz[i] - Yc[2]};
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) S[k + 3 * j] += xw[k] * yw[j];
    }
    double gap = 0, lmax = 0;
    FN(pose_update)(Xc, Yc, S, R, t, q_prev, &gap, &lmax);
    if (trace && iter < trace_cap)
      FN(trace_put)(trace + (size_t)ORACLE_TRACE_STRIDE * iter, iter, (double)iter, cost, Xc, Yc, S, R, t, gap,
                    lmax);
  }
  if (nn_out) memcpy(nn_out, nn, sizeof(int) * (size_t)M);
  free(nn);
  free(d2min);
  return maxIteration;
}

#undef FN
#undef CAT
#undef CAT_
