// Pose update of one Softassign inner iteration, shared by the matrix-free
// kernels (sm_103a): from the grid-reduced moments to the next pose
// (src/softassign.cu:772-798 then findRTfromS, src/findRTfromS.cpp:33-159).
#pragma once
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {

struct SaPoseScratch {
  float S[9], xcp[3], yd[3], xc[3], yc[3];
};

// The certified solve as a call of its own: one thread runs it while the
// block waits, and outside the kernel's inlined code it gets its own register
// allocation instead of the sweeps' spills.
static __device__ __noinline__ void horn_fast_call(const float* S, HornState<float>* st, float* q, float* gap,
                                                   float* lmax) {
  horn_quaternion_fast<float>(S, *st, q, gap, lmax);
}

// Block-wide (every thread calls it). s_tot: the 32 moments; s_hdr: oX, oY,
// mean(Y') (centring header). Threads 0..8 form S and threads 9..11 the
// centres; thread 0 then solves Horn's problem (warm-started eigenbasis in
// `horn`) and writes the next centred pose to s_pose. In the block that
// `leads`, it also writes the adjoint's record (tape_rec, kSaTape floats, when
// given), the trace record (trace_rec, 32 doubles, when given) and the step
// count. `fast` selects the certified inverse iteration (horn_quaternion_fast,
// no eigenbasis for an adjoint; the trace's gap is then -1) over the Jacobi
// solve that the taped kernels need.
__device__ __forceinline__ void sa_pose_update(const df* s_tot, const float* s_hdr, SaPoseScratch& ps,
                                               HornState<float>& horn, float* s_pose, bool leads,
                                               float* tape_rec, double* trace_rec, int step, float T,
                                               Ctl* ctl, Timeline* tl = nullptr, bool fast = false) {
  const int tid = threadIdx.x;
  if (tid < 12) sa_moments_to_S(tid, s_tot, &s_hdr[0], &s_hdr[3], &s_hdr[6], ps.S, ps.xcp, ps.yd, ps.xc, ps.yc);
  __syncthreads();
  if (tl) tl->mark(13);
  if (tid == 0) {
    const float* oX = &s_hdr[0];
    const float* oY = &s_hdr[3];
    float S[9], Xc[3], Yc[3], Xcp[3], Yd[3];
    for (int k = 0; k < 9; ++k) S[k] = ps.S[k];
    for (int i = 0; i < 3; ++i) {
      Xc[i] = ps.xc[i];
      Yc[i] = ps.yc[i];
      Xcp[i] = ps.xcp[i];
      Yd[i] = ps.yd[i];
    }
    float q[4], gap = 0.f, lmax = 0.f, Rn[9], tn[3];
    if (fast)
      horn_fast_call(S, &horn, q, &gap, &lmax);
    else
      horn_quaternion<float>(S, horn, q, &gap, &lmax);
    // centred-frame translation t' = Xc' - R (Yc - oY)
    quat_to_pose<float>(q, Xcp, Yd, Rn, tn);
    for (int k = 0; k < 9; ++k) s_pose[k] = Rn[k];
    for (int k = 0; k < 3; ++k) s_pose[9 + k] = tn[k];
    if (leads) {
      if (tape_rec) {  // the update's solve, for the adjoint
        tape_rec[12] = s_tot[0].hi;
        tape_rec[13] = s_tot[0].lo;
        for (int i = 0; i < 3; ++i) {
          tape_rec[14 + i] = Xc[i];
          tape_rec[17 + i] = Yc[i];
          tape_rec[20 + i] = Xcp[i];
          tape_rec[23 + i] = Yd[i];
        }
        for (int i = 0; i < 9; ++i) tape_rec[26 + i] = S[i];
        for (int i = 0; i < 4; ++i) tape_rec[35 + i] = q[i];
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) tape_rec[39 + 4 * i + j] = horn.V[i][j];
      }
      if (trace_rec) {
        double* rec = trace_rec;
        float to[3];
        pose_from_centred(Rn, tn, oX, oY, to);
        rec[0] = step;
        rec[1] = T;
        rec[2] = df_dbl(s_tot[0]);
        for (int i = 0; i < 3; ++i) {
          rec[3 + i] = Xc[i];
          rec[6 + i] = Yc[i];
          rec[27 + i] = to[i];
        }
        for (int k = 0; k < 9; ++k) {
          rec[9 + k] = S[k];
          rec[18 + k] = Rn[k];
        }
        rec[30] = gap;
        rec[31] = lmax;
      }
      ctl->steps_done = step + 1;
    }
  }
  __syncthreads();
}

}  // namespace cesa
