// Fused, streaming EM-ICP for sm_103a: the whole sigma schedule of emicp()
// (src/emicp.cu:441-669) in one persistent cooperative launch, with the N x M
// matrix A never materialised.
//
// Reference step (src/emicp.cu:453-635), rows r = Y points, columns c = X:
//   A_rc = exp(-|x_c - (R y_r + t)|^2 / sigma_p2)               (updateA)
//   C_r  = sum_c A_rc + exp(-d_02 / sigma_p2)                    (Sgemv + Saxpy)
//   A_rc <- sqrt(A_rc / C_r)   if C_r > 1e-6, else 1/N           (normalizeRowsOfA)
//   lambda_r = sum_c A_rc,  X'_r = sum_c A_rc x_c / lambda_r     (Sgemv, Sgemm, division)
//   Xc = sum lambda X' / sum lambda,  Yc = sum lambda y / sum lambda
//   S  = sum_r lambda_r (X'_r - Xc)(y_r - Yc)^T,  pose = findRTfromS(Xc, Yc, S)
// One-pass restatement used here: with e_rc = exp(-d^2 / (2 sigma_p2)) we have
// A = e^2 and sqrt(A / C) = e / sqrt(C). Per row, three running sums over the
// columns give everything: sum e^2, sum e, sum e*x. Then
//   C_r = sum e^2 + outlier,  lambda_r = sum e / sqrt(C_r),  lambda_r X'_r = sum e x / sqrt(C_r).
// Per element that is 3 FADD (direct differences), FMUL + 2 FFMA (d^2),
// FMUL (scale), 1 MUFU ex2, and FFMA + FADD + 3 FFMA (accumulators): 12 FP32
// pipe ops + 1 MUFU op. Large clouds take the ranged sweep on clouds scaled by
// sqrt(log2(e) / (2 sigma_p2)) (a scaled copy of X' per step), which drops the
// scale multiply: 11 FP32 ops.
//
// Coordinates are centred on the device (FP32 offsets oX, oY) before the
// loop. EM-ICP's S is translation invariant, so only Xc, Yc and t are shifted
// back; the pose enters and leaves in the caller's frame.
#include <atomic>
#include <cstdlib>

#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {

struct EmicpArgs {
  const float4* rows;  // Y' centred (owned), M
  const float4* cols;  // X' centred (streamed), N
  int M, N;
  SweepGeom geo;
  float sigma0, sigma_factor, d_02;
  int nsteps;
  const CenterHdr* hdr;
  float* dRt;           // PoseIO in/out, caller frame
  float* part;          // row partials [5][S][Mp] (accumulator, column slice, row); ranged: [5][nblk][kmax][128]
  float4* xs;           // ranged sweeps: X' scaled for the step, [2][N] by step parity
  int Mp;
  df* rbpart;           // [2][grid][kEmNV] moments per block (step parity)
  Ctl* ctl;
  unsigned* pair_tab;   // SM pairs (geo.pair_num): [2 kPairCap + 1], zero at launch
  float* pair_t;        // SM pairs: [grid] sweep time of each virtual block, ns
  double* trace;
  int trace_cap;
  float* row_out;       // optional [M][5] (centred-frame u)
  float* tape;          // optional [nsteps][kEmTape]
  float* row_tape;      // optional [nsteps][M][5]
  int* d_status;
  unsigned long long* tl;
  int tl_cap;
  uint64_t timeout_ns;
};

__global__ void __launch_bounds__(kThreads, 2) emicp_kernel(const EmicpArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SweepSmem& sm = *reinterpret_cast<SweepSmem*>(smem_raw);
  __shared__ float s_pose[12];
  __shared__ df s_red[kThreads];
  __shared__ OwnCache oc_rows;
  __shared__ RangedShare rs_rows;  // this block's share of a ranged sweep
  __shared__ int s_pair[3];        // SM pairs: pair index (-1: none), role, parts swapped
  __shared__ uint64_t s_tsweep;    // SM pairs: start of the step's sweep
  __shared__ df s_tot[kEmNV];
  __shared__ float s_emS[15];  // S, Xc, Yc of the step
  __shared__ float s_hdr[12];

  const int tid = threadIdx.x;
  const unsigned G = gridDim.x;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&sm.full[s], 1);
    mbar_init_fence();
    for (int k = 0; k < 3; ++k) {
      s_hdr[k] = A.hdr->oX[k];
      s_hdr[3 + k] = A.hdr->oY[k];
      s_hdr[6 + k] = A.hdr->xmean[k];
    }
    float R[9], t[3], tc[3];
    for (int k = 0; k < 9; ++k) R[k] = A.dRt[k];
    for (int k = 0; k < 3; ++k) t[k] = A.dRt[9 + k];
    pose_to_centred(R, t, &s_hdr[0], &s_hdr[3], tc);
    for (int k = 0; k < 9; ++k) s_pose[k] = R[k];
    for (int k = 0; k < 3; ++k) s_pose[9 + k] = tc[k];
    oc_rows.blk = -1;
    int vb = (int)blockIdx.x;  // the virtual block whose share this block sweeps
    s_pair[0] = -1;
    if (A.geo.pair_num) {
      const int2 pr = join_sm_pair(A.pair_tab, A.timeout_ns);
      if (pr.x >= 0 && pr.x < (int)G / 2) {
        s_pair[0] = pr.x;
        s_pair[1] = pr.y;
        s_pair[2] = 0;
        vb = 2 * pr.x + pr.y;
      } else {
        set_status(A.ctl, kStatusInternal, 23);  // the launch ends at its first grid barrier
      }
    }
    rs_rows = A.geo.pair_num && s_pair[0] < 0 ? RangedShare{0, -1, 0, 0, 0} : ranged_share(A.geo, vb, (int)G);
  }
  __syncthreads();

  __shared__ HornState<float> horn;       // the pose's solver state (thread 0)
  __shared__ HornState<float> horn_tape;  // block 0 with a tape: the eigenbasis for the adjoint
  if (tid == 0) {
    horn.reset();
    horn_tape.reset();
  }
  Pipe pipe;
  pipe_init(pipe);
  unsigned epoch = 0;
  const StreamSrc src{A.cols, nullptr, true};
  float s2 = A.sigma0;
  Timeline tl{A.tl, A.tl_cap, 0};
  // Ranged sweeps stream X' scaled by sc = sqrt(log2(e) / (2 s2)) (and scale the
  // owned rows alike), so that an element needs no scale of its own. Each step's
  // copy is written by all blocks during the previous step's row completion.
  auto scale_x = [&](float4* dst, float sc) {
    for (int i = (int)blockIdx.x * kThreads + tid; i < A.N; i += (int)G * kThreads) {
      const float4 x = ld_cg(A.cols + i);
      __stcg(dst + i, make_float4(x.x * sc, x.y * sc, x.z * sc, 0.f));
    }
  };
  bool started = true;  // false: the barrier after the first scaled copy gave up
  if (A.geo.ranged && A.nsteps > 0) {
    scale_x(A.xs, sqrtf(kLog2e / (2.f * s2)));
    started = grid_sync(A.ctl, epoch, G, A.timeout_ns, 22);
  }

  for (int step = 0; step < A.nsteps && started; ++step) {
    tl.mark(1);
    // the scaled X' was written by other blocks' ordinary stores, ahead of a
    // grid barrier; the bulk copies that stream it read through the async proxy
    if (A.geo.ranged && tid == 0) asm volatile("fence.proxy.async.global;" ::: "memory");
    const float outlier = expf(-A.d_02 / s2);  // src/emicp.cu:489
    float R[9], tc[3];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
    __syncthreads();

    // e = exp(-d2 / (2 s2)) = 2^(nk d2). Every unit stores its rows' partial
    // sums over its column slice (deferred: no completion counter).
    const float sc = sqrtf(kLog2e / (2.f * s2));
    if (A.geo.ranged) {
      float Rs[9], tcs[3];
#pragma unroll
      for (int k = 0; k < 9; ++k) Rs[k] = R[k] * sc;
#pragma unroll
      for (int k = 0; k < 3; ++k) tcs[k] = tc[k] * sc;
      const StreamSrc xsrc{A.xs + (size_t)(step & 1) * A.N, nullptr, false};
      if (tid == 0 && s_pair[0] >= 0) s_tsweep = global_ns();
      if (!sweep_units<5, EmicpElemScaled, NoPrep, NoFin, true, 1>(sm, pipe, A.geo, xsrc, A.rows, true, Rs, tcs, 0u,
                                                                A.part, nullptr, EmicpElemScaled{}, NoPrep{}, NoFin{},
                                                                A.ctl, A.timeout_ns, 10, tl, A.Mp, &oc_rows, &rs_rows))
        break;
      if (tid == 0 && s_pair[0] >= 0)
        A.pair_t[2 * s_pair[0] + (s_pair[1] ^ s_pair[2])] = (float)(global_ns() - s_tsweep);
    } else {
      const EmicpElem elem{-kLog2e / (2.f * s2)};
      if (!sweep_units<5, EmicpElem, NoPrep, NoFin, true, 0>(sm, pipe, A.geo, src, A.rows, true, R, tc, 0u, A.part,
                                                           nullptr, elem, NoPrep{}, NoFin{}, A.ctl, A.timeout_ns, 10,
                                                           tl, A.Mp, &oc_rows))
        break;
    }
    if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, 20)) break;
    tl.mark(5);
    if (tid == 0 && s_pair[0] >= 0) {  // SM pairs: the parts change blocks when the times show the other favoured
      long lo = 0, sp = 0, hi = 0;
      ranged_tasks(A.geo, 2 * s_pair[0], (int)G, lo, sp);
      ranged_tasks(A.geo, 2 * s_pair[0] + 1, (int)G, sp, hi);
      if (pair_swap(lo, sp, hi, A.pair_t, s_pair[0])) {
        s_pair[2] ^= 1;
        rs_rows = ranged_share(A.geo, 2 * s_pair[0] + (s_pair[1] ^ s_pair[2]), (int)G);
      }
    }
    // the next step's scaled X' (its buffer was last read by the previous step's sweep)
    if (A.geo.ranged && step + 1 < A.nsteps)
      scale_x(A.xs + (size_t)((step + 1) & 1) * A.N, sqrtf(kLog2e / (2.f * (s2 * A.sigma_factor))));

    // ---- rows completed, each block a contiguous share of them; its 16
    // moments are one record. Thread t first sums the slice partials of
    // (row, accumulator) pairs t, t + kThreads, ... (loads in flight together),
    // then row threads finish their rows (emicp_row_finish).
    df* rb = A.rbpart + (size_t)(step & 1) * G * kEmNV;
    {
      const int S = A.geo.slices;
      const float inv_sc = 1.f / sc;
      const int rpc = (A.M + (int)G - 1) / (int)G;
      const int r0 = (int)blockIdx.x * rpc;
      const int nrows = max(0, min(rpc, A.M - r0));
      float* stot = reinterpret_cast<float*>(&sm.raw2[0][0]);  // [kThreads][5]; raw2 carries no stream here
      static_assert(sizeof(sm.raw2) >= sizeof(float) * 5 * kThreads, "row sums scratch");
      static_assert(offsetof(SweepSmem, full) - offsetof(SweepSmem, prep) >= sizeof(df) * (kEmNV + 1) * kThreads,
                    "moment scratch");
      const float xm[3] = {s_hdr[6], s_hdr[7], s_hdr[8]};
      const float oX[3] = {s_hdr[0], s_hdr[1], s_hdr[2]};
      float* row_tape = A.row_tape ? A.row_tape + (size_t)step * A.M * 5 : nullptr;
      df v[kEmNV];
#pragma unroll
      for (int k = 0; k < kEmNV; ++k) v[k] = df_make(0.f);
      for (int c0 = 0; c0 < nrows; c0 += kThreads) {  // rows [c0, c0 + kThreads) of the share
        const int nr = min(kThreads, nrows - c0);
        for (int pq = tid; pq < 5 * nr; pq += kThreads) {
          const int a = pq % 5, rr = pq / 5;
          if (A.geo.ranged) {  // the kmax slots of the row's owned block, in task order
            const int kmax = A.geo.kmax;
            const float* P = A.part + (size_t)a * A.geo.nblk * kmax * kBlockPts + ranged_slot0(r0 + c0 + rr, kmax);
            float sum = 0.f;
            for (int j = 0; j < kmax; j += 4) {  // 4 loads in flight, then added in slot order
              float w[4];
#pragma unroll
              for (int q = 0; q < 4; ++q) w[q] = j + q < kmax ? __ldcg(P + (size_t)(j + q) * kBlockPts) : 0.f;
#pragma unroll
              for (int q = 0; q < 4; ++q) sum += w[q];
            }
            stot[rr * 5 + a] = a >= 2 ? sum * inv_sc : sum;  // the scaled coordinates' sums
            continue;
          }
          const float* P = A.part + (size_t)a * S * A.Mp + r0 + c0 + rr;
          float sum = 0.f;
          int k = 0;
          for (; k + 16 <= S; k += 16) {
            float w[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) w[j] = __ldcg(P + (size_t)(k + j) * A.Mp);
#pragma unroll
            for (int j = 0; j < 16; ++j) sum += w[j];
          }
          if (k < S) {
            float w[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) w[j] = k + j < S ? __ldcg(P + (size_t)(k + j) * A.Mp) : 0.f;
#pragma unroll
            for (int j = 0; j < 16; ++j) sum += w[j];  // adding the zeros leaves the sum unchanged
          }
          stot[rr * 5 + a] = sum;
        }
        __syncthreads();
        if (tid < nr) {
          const int r = r0 + c0 + tid;
          const float tot[5] = {stot[tid * 5], stot[tid * 5 + 1], stot[tid * 5 + 2], stot[tid * 5 + 3],
                                stot[tid * 5 + 4]};
          emicp_row_finish(r, tot, ld_cg(A.rows + r), outlier, xm, A.row_out, oX, row_tape, v);
        }
        __syncthreads();
      }
      em_block_moments(v, min(nrows, kThreads), reinterpret_cast<df*>(sm.prep), rb + (size_t)blockIdx.x * kEmNV);
    }
    if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, 21)) break;
    tl.mark(8);

    // ---- grid-wide moments -> pose (every block computes the same pose)
    reduce_block_partials<kEmNV>(rb, (int)G, s_red, s_tot);
    tl.mark(6);
    em_moments_to_S_block(s_tot, s_emS);
    if (tid == 0) {
      float Xc[3], Yc[3], S[9];
      for (int k = 0; k < 9; ++k) S[k] = s_emS[k];
      for (int k = 0; k < 3; ++k) {
        Xc[k] = s_emS[9 + k];
        Yc[k] = s_emS[12 + k];
      }
      float q[4], gap = 0.f, lmax = 0.f, Rn[9], tn[3];
      // the pose: certified inverse iteration (Jacobi fallback); the same with
      // and without a tape, so that both forwards agree bitwise
      horn_quaternion_fast<float>(S, horn, q, &gap, &lmax);
      quat_to_pose<float>(q, Xc, Yc, Rn, tn);
      if (A.tape && blockIdx.x == 0) {  // the step's inputs and solve for the adjoint
        // the adjoint's eigenbasis, from a Jacobi solve of the same S on its own
        // state (it does not feed back into the pose)
        float qj[4], gj = 0.f, lj = 0.f;
        horn_quaternion<float>(S, horn_tape, qj, &gj, &lj);
        float* rec = A.tape + (size_t)step * kEmTape;
        for (int k = 0; k < 12; ++k) rec[k] = s_pose[k];
        rec[12] = s2;
        for (int k = 0; k < kEmNV; ++k) {
          rec[16 + 2 * k] = s_tot[k].hi;
          rec[17 + 2 * k] = s_tot[k].lo;
        }
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) rec[48 + 4 * i + j] = horn_tape.V[i][j];
        for (int k = 0; k < 4; ++k) rec[64 + k] = q[k];
      }
      for (int k = 0; k < 9; ++k) s_pose[k] = Rn[k];
      for (int k = 0; k < 3; ++k) s_pose[9 + k] = tn[k];
      if (blockIdx.x == 0) {
        if (A.trace && step < A.trace_cap) {
          double* rec = A.trace + (size_t)step * 32;
          float to[3];
          pose_from_centred(Rn, tn, &s_hdr[0], &s_hdr[3], to);
          rec[0] = step;
          rec[1] = s2;
          rec[2] = df_dbl(s_tot[0]);
          for (int i = 0; i < 3; ++i) {
            rec[3 + i] = (double)Xc[i] + (double)s_hdr[i];
            rec[6 + i] = (double)Yc[i] + (double)s_hdr[3 + i];
            rec[27 + i] = to[i];
          }
          for (int k = 0; k < 9; ++k) {
            rec[9 + k] = S[k];
            rec[18 + k] = Rn[k];
          }
          rec[30] = gap;
          rec[31] = lmax;
        }
        A.ctl->steps_done = step + 1;
      }
    }
    __syncthreads();
    tl.mark(7);
    s2 *= A.sigma_factor;  // FP32, src/emicp.cu:668
  }

  if (blockIdx.x == 0 && tid == 0) {
    const int st = ld_status(A.ctl);
    if (st == kStatusOk) {
      float R[9], tc[3], t[3];
      for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
      for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
      pose_from_centred(R, tc, &s_hdr[0], &s_hdr[3], t);
      for (int k = 0; k < 9; ++k) A.dRt[k] = R[k];
      for (int k = 0; k < 3; ++k) A.dRt[9 + k] = t[k];
    }
    if (A.d_status) *A.d_status = st;
    if (A.tl) A.ctl->pad[0] = (unsigned)tl.n;
  }
}

// ------------------------------------------------------------------ host side

namespace {
struct Carve {
  char* p;
  size_t off = 0;
  explicit Carve(void* base) : p(static_cast<char*>(base)) {}
  template <class T>
  T* take(size_t n) {
    off = (off + 255) & ~size_t(255);
    T* r = p ? reinterpret_cast<T*>(p + off) : nullptr;
    off += n * sizeof(T);
    return r;
  }
};

struct EmicpPlan {
  int grid;
  SweepGeom geo;
  size_t smem;
};

size_t sweep_smem() { return sizeof(SweepSmem); }

EmicpPlan plan_emicp(int N, int M, int device) {
  EmicpPlan P;
  P.smem = sweep_smem();
  const int limit = persistent_grid_limit(device, (const void*)emicp_kernel, P.smem);
  const SweepGeomH h = plan_sweep(M, N, limit);
  P.geo = SweepGeom{h.n_own, h.n_stream, h.nblk, h.slices, h.slice_len, h.units, 0, 0, 0, 0};
  P.grid = h.units < limit ? h.units : limit;
  // Large clouds: contiguous task ranges, the same work per block to one
  // chunk of 512 streamed points, instead of units dealt in waves; with two
  // blocks on every SM, each SM's pair splits its range 13 : 3, the larger
  // part to the block the SM favours.
  if (ranged_pays(h.nblk, N, limit)) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const char* ev = getenv("CESA_SM_PAIRS");  // "0": equal shares (for comparisons)
    if (sms > 0 && limit == 2 * sms && !(ev && ev[0] == '0')) P.geo.pair_num = 208;  // 13 / 16
    make_ranged(P.geo, limit);
    P.grid = limit;
  }
  return P;
}

struct EmicpCarved {
  Ctl* ctl;
  CenterHdr* hdr;
  float4* rows;
  float4* cols;
  float4* xs;
  float* part;
  df* rbpart;
  unsigned* pair_tab;
  float* pair_t;
  int Mp;
};

EmicpCarved carve_emicp(void* base, const EmicpPlan& P, int N, int M, size_t* total) {
  Carve c(base);
  EmicpCarved w;
  w.Mp = (M + 3) & ~3;
  w.ctl = c.take<Ctl>(1);
  w.hdr = c.take<CenterHdr>(1);
  w.rows = c.take<float4>((size_t)M);
  w.cols = c.take<float4>((size_t)N);
  w.xs = c.take<float4>(P.geo.ranged ? (size_t)2 * N : 0);
  w.part = c.take<float>(P.geo.ranged ? (size_t)5 * P.geo.nblk * P.geo.kmax * kBlockPts
                                      : (size_t)5 * P.geo.slices * w.Mp);
  w.rbpart = c.take<df>((size_t)2 * P.grid * kEmNV);
  w.pair_tab = c.take<unsigned>(P.geo.pair_num ? 2 * kPairCap + 1 : 0);
  w.pair_t = c.take<float>(P.geo.pair_num ? (size_t)P.grid : 0);
  if (total) *total = c.off;
  return w;
}
}  // namespace

void emicp_ws_views(void* ws, int N, int M, int device, CenterHdr** hdr, float4** rows, float4** cols) {
  const EmicpPlan P = plan_emicp(N, M, device);
  EmicpCarved w = carve_emicp(ws, P, N, M, nullptr);
  *hdr = w.hdr;
  *rows = w.rows;
  *cols = w.cols;
}

size_t emicp_ws_need(int N, int M, int device) {
  const EmicpPlan P = plan_emicp(N, M, device);
  size_t total = 0;
  carve_emicp(nullptr, P, N, M, &total);
  return total;
}

int enqueue_emicp(const EmicpLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  const EmicpPlan P = plan_emicp(L.N, L.M, device);
  size_t total = 0;
  EmicpCarved w = carve_emicp(ws, P, L.N, L.M, &total);
  if (total > ws_bytes) return (int)cudaErrorInvalidValue;
  if (grid_used) *grid_used = P.grid;
  // the control block starts at zero every launch, and so do the ranged
  // partial slots (those no block writes must read as zero)
  e = cudaMemsetAsync(w.ctl, 0, sizeof(Ctl), st);
  if (e == cudaSuccess && P.geo.ranged)
    e = cudaMemsetAsync(w.part, 0, sizeof(float) * 5 * (size_t)P.geo.nblk * P.geo.kmax * kBlockPts, st);
  if (e == cudaSuccess && P.geo.pair_num)
    e = cudaMemsetAsync(w.pair_tab, 0, sizeof(unsigned) * (2 * kPairCap + 1), st);
  if (e != cudaSuccess) return (int)e;
  prep_center_kernel<<<1, 1024, 0, st>>>(L.dX, L.N, L.dY, L.M, w.hdr);
  const int pb = 256, pg_x = (L.N + pb - 1) / pb, pg_y = (L.M + pb - 1) / pb;
  prep_pack_kernel<<<pg_x < 1024 ? pg_x : 1024, pb, 0, st>>>(L.dX, L.N, w.hdr, 0, 0.f, w.cols);
  prep_pack_kernel<<<pg_y < 1024 ? pg_y : 1024, pb, 0, st>>>(L.dY, L.M, w.hdr, 1, 0.f, w.rows);
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (L.nsteps <= 0) return 0;

  EmicpArgs A;
  A.rows = w.rows;
  A.cols = w.cols;
  A.M = L.M;
  A.N = L.N;
  A.geo = P.geo;
  A.sigma0 = L.sigma_p2;
  A.sigma_factor = L.sigma_factor;
  A.d_02 = L.d_02;
  A.nsteps = L.nsteps;
  A.hdr = w.hdr;
  A.dRt = L.dRt;
  A.part = w.part;
  A.xs = w.xs;
  A.Mp = w.Mp;
  A.rbpart = w.rbpart;
  A.ctl = w.ctl;
  A.pair_tab = w.pair_tab;
  A.pair_t = w.pair_t;
  A.trace = L.trace;
  A.trace_cap = L.trace_cap;
  A.row_out = L.row_out;
  A.tape = L.tape;
  A.row_tape = L.row_tape;
  A.d_status = L.d_status;
  A.tl = L.timeline;
  A.tl_cap = L.timeline_cap;
  A.timeout_ns = L.timeout_ns;
  void* args[] = {(void*)&A};
  e = cudaLaunchCooperativeKernel((const void*)emicp_kernel, dim3(P.grid), dim3(kThreads), args,
                                  P.smem, st);
  return (int)e;
}

int read_ws_status(void* ws, cudaStream_t st, int* status, int* steps, int* tl_written) {
  Ctl h;
  cudaError_t e = cudaMemcpyAsync(&h, ws, sizeof(Ctl), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return (int)e;
  if (status) *status = h.status;
  if (steps) *steps = h.steps_done;
  if (tl_written) *tl_written = (int)h.pad[0];
  return 0;
}

// Smem opt-in and occupancy for a persistent kernel: blocks per SM x SMs.
int persistent_grid_limit(int device, const void* kernel, size_t smem) {
  // SM count per device, filled on first use; each entry is written once with
  // its device's own value, so concurrent callers on other devices cannot mix
  // them up.
  static std::atomic<int> sms_of[64];
  int sms = 0;
  if (device >= 0 && device < 64) sms = sms_of[device].load(std::memory_order_relaxed);
  if (sms <= 0) {
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (device >= 0 && device < 64 && sms > 0) sms_of[device].store(sms, std::memory_order_relaxed);
  }
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, smem);
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 2) per_sm = 2;
  return per_sm * (sms > 0 ? sms : 1);
}

// Unit decomposition over the split S. Modelled time, in element
// evaluations of one block (~20 per ns): waves x (unit work + fixed cost per
// unit: streamed-chunk latency, reductions) + the completion of split owned
// blocks (partials written, the last unit loads S partials per accumulator,
// 16 in flight).
SweepGeomH plan_sweep(int n_own, int n_stream, int grid_limit) {
  SweepGeomH best{};
  const int nblk = (n_own + kBlockPts - 1) / kBlockPts;
#ifndef CESA_UNIT_FIXED_COST
#define CESA_UNIT_FIXED_COST 40000.0  // per-unit cost in element evaluations of one block
#endif
  const double fixed = CESA_UNIT_FIXED_COST;
  double best_cost = 1e300;
  const int smax_stream = (n_stream + 31) / 32;
  const int smax = smax_stream < 128 ? smax_stream : 128;
  for (int S = 1; S <= (smax > 0 ? smax : 1); ++S) {
    const int slice_len = (n_stream + S - 1) / S;
    const int s_eff = (n_stream + slice_len - 1) / slice_len;
    if (s_eff != S) continue;
    const long units = (long)nblk * S;
    const int grid = units < grid_limit ? (int)units : grid_limit;
    const long waves = (units + grid - 1) / grid;
    const double split = S > 1 ? 30000.0 + 15000.0 * ((S + 15) / 16) : 0.0;
    const double cost = (double)waves * ((double)kBlockPts * slice_len + fixed) + split;
    if (cost < best_cost * 0.999) {
      best_cost = cost;
      best = SweepGeomH{n_own, n_stream, nblk, S, slice_len, (int)units};
    }
  }
  if (best.units == 0) best = SweepGeomH{n_own, n_stream, nblk, 1, n_stream, nblk};
  return best;
}

}  // namespace cesa
