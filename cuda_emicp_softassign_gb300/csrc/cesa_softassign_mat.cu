// Softassign with the materialised Sinkhorn form, for sm_103a: the whole
// annealing schedule of softassign() (src/softassign.cu:486-822) in one
// persistent cooperative launch, with the affinity matrix K stored once per
// pose update and the Sinkhorn passes streaming it from HBM.
//
// Per pose update (T, R, t fixed):
//   W   (= row pass 0) computes K_rc = exp((alpha - |x_r - (R y_c + t)|^2)/T)/sqrt(T)
//       exactly as the matrix-free sweep does, stores it, and sums its rows;
//   C_k column pass k:  cs = b_old (K^T a) + u_old, b = b_old / cs, u = u_old / cs;
//   R_k row pass k >= 1: rs = a_old (K b) + s_old,  a = a_old / rs,  s = s_old / rs;
//   F   final pass: w = a (K b), mu = a (K delta), Vhat = a (K g (y' - Yhat)),
//       then the 28 row moments, the 4 column moments of the last column pass,
//       S and Horn's pose (the same moment algebra as the matrix-free kernel).
// Bytes per affinity element and pose update: 4 written by W, 4 read by each
// of the 2*I1 later passes (28 at I1 = 3). K uses the tiled layout
// K[row block][column][128 rows]: a column of a row block is 512 contiguous
// bytes, so W stores whole 128-byte lines per warp, and every later pass
// streams contiguous 16 KiB sub-blocks (32 columns x 128 rows) through a
// three-stage TMA ring. Row passes own 128 rows (4 per lane) and sum their
// columns in registers; column passes own 128 columns (16 per warp) and sum
// each column across the lanes. Every pass completes its owned blocks by
// arrival counter over the slices (split completion).
#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {
namespace {

constexpr int kSubCols = 32;                       // columns per K sub-block
constexpr int kSubFloats = kSubCols * kBlockPts;   // 16 KiB
constexpr int kMStages = 3;
constexpr int kColsPerWarp = kBlockPts / kWarps;   // 16 owned columns per warp in a column pass

struct __align__(16) MatSmem {
  // raw .. red is one contiguous region, also the moment scratch of the final pass
  float4 raw[2][kChunk];  // W: streamed Y' chunks
  float4 prep[kChunk];    // W: posed chunk
  float red[kMaxAcc][kWarps][kBlockPts];
  float kb[kMStages][kSubFloats];       // K sub-blocks
  float wb[kMStages][5][kSubCols];      // row passes: weights of the sub-block's columns
  float ab[kMStages][kBlockPts];        // column passes: a of the sub-block's row block
  float colsum[kBlockPts];
  uint64_t kfull[kMStages];
  uint64_t full[2];
  int flag;
};
static_assert(offsetof(MatSmem, kb) - offsetof(MatSmem, raw) >= 32 * (kBlockPts + 8) * sizeof(df),
              "moment scratch does not fit");

struct MatArgs {
  const float4* rows;  // X' centred (N)
  const float4* cols;  // Y' centred (M)
  float* K;            // [nblk_r][M][128]
  float *a, *s, *rs;   // [nblk_r * 128], zero beyond N
  float *b, *u, *cs;   // [Mp]
  float* w5;           // [5][Mp] final-pass column weights: b, delta, g (y' - Yhat)
  float* w_out;        // optional [N]: final row sums w of the last pose update
  int N, M, Mp;
  SweepGeom gr;  // row passes: own row blocks, slices of columns (multiples of kSubCols)
  SweepGeom gc;  // column passes: own column blocks, slices of row blocks
  int JMAX, I0, I1;
  float alpha, T0, TFACTOR;
  const CenterHdr* hdr;
  float* dRt;
  float* part;
  unsigned* cnt_r;
  unsigned* cnt_c;
  df* rec;  // [nblk_r + nblk_c][32]
  Ctl* ctl;
  double* trace;
  int trace_cap;
  int* d_status;
  uint64_t timeout_ns;
};

// ---------------------------------------------------------------- K sub-block ring
struct SubTask {
  const float* k;    // first float of the sub-block
  int ncols;         // columns in it (<= kSubCols), 0 = none
  const float* w[5]; // row passes: weights of its first column (nw arrays)
  int nw;
  const float* a;    // column passes: a of its row block (128 floats)
};

struct KRing {
  unsigned uses[kMStages];
  int next;
};

__device__ __forceinline__ int kring_issue(KRing& rg, MatSmem& sm, const SubTask& t, unsigned& par) {
  const int st = rg.next;
  rg.next = (rg.next + 1) % kMStages;
  rg.uses[st] += 1;
  par = (rg.uses[st] - 1u) & 1u;
  if (threadIdx.x == 0) {
    const unsigned kbytes = (unsigned)t.ncols * kBlockPts * 4u;
    const unsigned wbytes = (unsigned)((t.ncols + 3) & ~3) * 4u;
    const unsigned total = kbytes + (unsigned)t.nw * wbytes + (t.a ? kBlockPts * 4u : 0u);
    mbar_arrive_expect_tx(&sm.kfull[st], total);
    bulk_g2s(&sm.kb[st][0], t.k, kbytes, &sm.kfull[st]);
    for (int i = 0; i < t.nw; ++i) bulk_g2s(&sm.wb[st][i][0], t.w[i], wbytes, &sm.kfull[st]);
    if (t.a) bulk_g2s(&sm.ab[st][0], t.a, kBlockPts * 4u, &sm.kfull[st]);
  }
  return st;
}

// Sub-block i of a row-pass unit (row block rb, columns [c_begin, c_end)).
__device__ __forceinline__ SubTask row_task(const MatArgs& A, int rb, int c_begin, int c_end, int i,
                                            const float* const* w, int nw) {
  SubTask t{};
  const int c0 = c_begin + i * kSubCols;
  if (c0 >= c_end) return t;
  t.ncols = min(kSubCols, c_end - c0);
  t.k = A.K + ((size_t)rb * A.M + c0) * kBlockPts;
  t.nw = nw;
  for (int q = 0; q < nw; ++q) t.w[q] = w[q] + c0;
  return t;
}

// Sub-blocks per row block of column block cb (the last block may be partial).
__device__ __forceinline__ int col_subs(const MatArgs& A, int cb) {
  return (min(kBlockPts, A.M - cb * kBlockPts) + kSubCols - 1) / kSubCols;
}

// Sub-block i of a column-pass unit (column block cb, row blocks [r_begin, r_end),
// nq sub-blocks per row block): row block r_begin + i / nq, columns
// cb*128 + 32 (i % nq) ...
__device__ __forceinline__ SubTask col_task(const MatArgs& A, int cb, int r_begin, int r_end, int nq, int i) {
  SubTask t{};
  const int rb = r_begin + i / nq;
  const int c0 = cb * kBlockPts + (i % nq) * kSubCols;
  if (rb >= r_end) return t;
  t.ncols = min(kSubCols, A.M - c0);
  t.k = A.K + ((size_t)rb * A.M + c0) * kBlockPts;
  t.a = A.a + (size_t)rb * kBlockPts;
  return t;
}

// ---------------------------------------------------------------- finalizers
struct MatRowFin {  // rs = a_old (K b) + s_old, a = a_old / rs, s = s_old / rs
  float *a, *s, *rs;
  int N;
  bool first;
  __device__ __forceinline__ void operator()(int blk, const float (&tot)[1]) const {
    const int r = blk * kBlockPts + (int)threadIdx.x;
    if (threadIdx.x < kBlockPts && r < N) {
      const float ao = first ? 1.f : __ldcg(a + r);
      const float so = __ldcg(s + r);
      const float rsv = fmaf(ao, tot[0], so);
      __stcg(a + r, ao / rsv);
      __stcg(s + r, so / rsv);
      __stcg(rs + r, rsv);
    }
  }
};

// cs = b_old (K^T a) + u_old, b = b_old / cs, u = u_old / cs. After the last
// column pass also the final-pass weights (b, delta = b (cs - 1), g (y' - Yhat)
// with g = b cs) and the column moments sum cs, sum cs y' (record slots 28..31).
struct MatColFin {
  float *b, *u, *cs, *w5;
  int M, Mp;
  bool first, last;
  const float4* cols;
  float yh[3];
  df* scratch;
  df* rec;
  __device__ __forceinline__ void operator()(int blk, const float (&tot)[1]) const {
    const int c = blk * kBlockPts + (int)threadIdx.x;
    const bool mine = threadIdx.x < kBlockPts && c < M;
    float csv = 0.f;
    float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
    if (mine) {
      const float bo = first ? 1.f : __ldcg(b + c);
      const float uo = __ldcg(u + c);
      csv = fmaf(bo, tot[0], uo);
      const float bn = bo / csv;
      __stcg(b + c, bn);
      __stcg(u + c, uo / csv);
      __stcg(cs + c, csv);
      if (last) {
        y = __ldcg(cols + c);
        const float g = bn * csv;
        __stcg(w5 + c, bn);
        __stcg(w5 + (size_t)Mp + c, bn * (csv - 1.f));
        __stcg(w5 + 2 * (size_t)Mp + c, g * (y.x - yh[0]));
        __stcg(w5 + 3 * (size_t)Mp + c, g * (y.y - yh[1]));
        __stcg(w5 + 4 * (size_t)Mp + c, g * (y.z - yh[2]));
      }
    }
    if (!last) return;  // uniform
    df v[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) v[k] = df_make(0.f);
    if (mine) {
      df_add(v[28], csv);
      df_add_prod(v[29], csv, y.x);
      df_add_prod(v[30], csv, y.y);
      df_add_prod(v[31], csv, y.z);
    }
    owned_block_sum<32>(v, scratch, rec + (size_t)blk * 32);
  }
};

// ---------------------------------------------------------------- passes
// W: K for the unit's 128 rows x its column slice, stored, and the row sums
// of K (b = 1). The streamed Y' chunks go through the two-stage ring raw[].
__device__ bool pass_write(MatSmem& sm, const MatArgs& A, unsigned round, const float (&R)[9],
                           const float (&tc)[3], float nk, float c0, unsigned (&uses)[2]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const SweepGeom& g = A.gr;
  for (int u = blockIdx.x; u < g.units; u += gridDim.x) {
    const int rb = u / g.slices, sl = u - rb * g.slices;
    const int cb = sl * g.slice_len, ce = min(cb + g.slice_len, A.M);
    float p[kOwnPerLane][3];
    bool valid[kOwnPerLane];
    {
      float4 ow[kOwnPerLane];
      load_owned(A.rows, A.N, rb, ow, valid);
#pragma unroll
      for (int j = 0; j < kOwnPerLane; ++j) {
        p[j][0] = ow[j].x;
        p[j][1] = ow[j].y;
        p[j][2] = ow[j].z;
      }
    }
    float2 q[kPairs][3];
    pack_owned(p, q);
    float2 acc[kPairs][1];
#pragma unroll
    for (int k = 0; k < kPairs; ++k) acc[k][0] = make_float2(0.f, 0.f);
    float* Kb = A.K + (size_t)rb * A.M * kBlockPts;
    // first chunk
    int st = 0;
    {
      uses[0] += 1;
      if (threadIdx.x == 0) {
        const int len = min(kChunk, ce - cb);
        mbar_arrive_expect_tx(&sm.full[0], (unsigned)len * 16u);
        bulk_g2s(&sm.raw[0][0], A.cols + cb, (unsigned)len * 16u, &sm.full[0]);
      }
    }
    for (int first = cb; first < ce; first += kChunk) {
      const int len = min(kChunk, ce - first);
      const int nst = st ^ 1;
      const bool more = first + kChunk < ce;
      if (more) {
        uses[nst] += 1;
        if (threadIdx.x == 0) {
          const int nlen = min(kChunk, ce - first - kChunk);
          mbar_arrive_expect_tx(&sm.full[nst], (unsigned)nlen * 16u);
          bulk_g2s(&sm.raw[nst][0], A.cols + first + kChunk, (unsigned)nlen * 16u, &sm.full[nst]);
        }
      }
      const bool bad = !mbar_wait(&sm.full[st], (uses[st] - 1u) & 1u, A.ctl, A.timeout_ns, 80);
      if (__syncthreads_or(bad)) {
        if (more) mbar_wait(&sm.full[nst], (uses[nst] - 1u) & 1u, A.ctl, A.timeout_ns, 81);
        return false;
      }
      for (int c = threadIdx.x; c < len; c += kThreads) {
        const float4 y = sm.raw[st][c];
        sm.prep[c] = make_float4(R[0] * y.x + R[1] * y.y + R[2] * y.z + tc[0],
                                 R[3] * y.x + R[4] * y.y + R[5] * y.z + tc[1],
                                 R[6] * y.x + R[7] * y.y + R[8] * y.z + tc[2], 1.f);
      }
      __syncthreads();
#pragma unroll 2
      for (int c = warp; c < len; c += kWarps) {
        const float4 y = sm.prep[c];
        float* kc = Kb + (size_t)(first + c) * kBlockPts;
#pragma unroll
        for (int k = 0; k < kPairs; ++k) {
          const float2 e = ex2_pair(__ffma2_rn(dist2_pair(q[k], y), dup2(nk), dup2(c0)));
          acc[k][0] = __fadd2_rn(acc[k][0], e);  // weight 1: the same as fmaf(e, 1, acc)
          kc[lane + 64 * k] = valid[2 * k] ? e.x : 0.f;
          kc[lane + 64 * k + 32] = valid[2 * k + 1] ? e.y : 0.f;
        }
      }
      __syncthreads();
      st = nst;
    }
    float tot[1];
    reduce_warps<1>(sm, acc, tot);
    if (split_complete<1>(sm, g, rb, sl, round, A.part, A.cnt_r, tot))
      MatRowFin{A.a, A.s, A.rs, A.N, true}(rb, tot);
  }
  return true;
}

// R_k (nw = 1, weights b) or F (nw = 5, weights w5): sums over the unit's
// columns of K times the column weights, for the unit's 128 rows.
template <int NW, class Fin>
__device__ bool pass_rows(MatSmem& sm, KRing& rg, const MatArgs& A, unsigned round, const float* const* w,
                          const Fin& fin) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const SweepGeom& g = A.gr;
  for (int u = blockIdx.x; u < g.units; u += gridDim.x) {
    const int rb = u / g.slices, sl = u - rb * g.slices;
    const int cb = sl * g.slice_len, ce = min(cb + g.slice_len, A.M);
    float acc[kOwnPerLane][NW];
#pragma unroll
    for (int j = 0; j < kOwnPerLane; ++j)
#pragma unroll
      for (int v = 0; v < NW; ++v) acc[j][v] = 0.f;
    int stq[kMStages];
    unsigned paq[kMStages];
    int issued = 0;
    for (; issued < kMStages - 1; ++issued) {
      const SubTask t = row_task(A, rb, cb, ce, issued, w, NW);
      if (!t.ncols) break;
      stq[issued % kMStages] = kring_issue(rg, sm, t, paq[issued % kMStages]);
    }
    for (int i = 0;; ++i) {
      const SubTask cur = row_task(A, rb, cb, ce, i, w, NW);
      if (!cur.ncols) break;
      const SubTask nt = row_task(A, rb, cb, ce, issued, w, NW);
      if (nt.ncols) {
        stq[issued % kMStages] = kring_issue(rg, sm, nt, paq[issued % kMStages]);
        ++issued;
      }
      const int st = stq[i % kMStages];
      const bool bad = !mbar_wait(&sm.kfull[st], paq[i % kMStages], A.ctl, A.timeout_ns, 82);
      if (__syncthreads_or(bad)) {
        for (int j = i + 1; j < issued; ++j) mbar_wait(&sm.kfull[stq[j % kMStages]], paq[j % kMStages], A.ctl,
                                                       A.timeout_ns, 83);
        return false;
      }
      const float* kb = sm.kb[st];
#pragma unroll
      for (int c4 = 0; c4 < kSubCols / kWarps; ++c4) {
        const int c = warp + kWarps * c4;
        if (c < cur.ncols) {
          float wv[NW];
#pragma unroll
          for (int v = 0; v < NW; ++v) wv[v] = sm.wb[st][v][c];
#pragma unroll
          for (int j = 0; j < kOwnPerLane; ++j) {
            const float kv = kb[c * kBlockPts + lane + 32 * j];
#pragma unroll
            for (int v = 0; v < NW; ++v) acc[j][v] = fmaf(kv, wv[v], acc[j][v]);
          }
        }
      }
      __syncthreads();
    }
    float tot[NW];
    reduce_warps<NW>(sm, acc, tot);
    if (split_complete<NW>(sm, g, rb, sl, round, A.part, A.cnt_r, tot)) fin(rb, tot);
  }
  return true;
}

// C_k: column sums of K times a over the unit's row blocks, for its 128
// columns; warp w owns columns w + 8 i (i < 16) and sums each across lanes.
__device__ bool pass_cols(MatSmem& sm, KRing& rg, const MatArgs& A, unsigned round, const MatColFin& fin0) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const SweepGeom& g = A.gc;
  for (int u = blockIdx.x; u < g.units; u += gridDim.x) {
    const int cbk = u / g.slices, sl = u - cbk * g.slices;
    const int rbeg = sl * g.slice_len, rend = min(rbeg + g.slice_len, g.n_stream);
    const int nq = col_subs(A, cbk);
    float acc[kColsPerWarp];
#pragma unroll
    for (int i = 0; i < kColsPerWarp; ++i) acc[i] = 0.f;
    int stq[kMStages];
    unsigned paq[kMStages];
    int issued = 0;
    for (; issued < kMStages - 1; ++issued) {
      const SubTask t = col_task(A, cbk, rbeg, rend, nq, issued);
      if (!t.ncols) break;
      stq[issued % kMStages] = kring_issue(rg, sm, t, paq[issued % kMStages]);
    }
    for (int i = 0;; ++i) {
      const SubTask cur = col_task(A, cbk, rbeg, rend, nq, i);
      if (!cur.ncols) break;
      const SubTask nt = col_task(A, cbk, rbeg, rend, nq, issued);
      if (nt.ncols) {
        stq[issued % kMStages] = kring_issue(rg, sm, nt, paq[issued % kMStages]);
        ++issued;
      }
      const int st = stq[i % kMStages];
      const bool bad = !mbar_wait(&sm.kfull[st], paq[i % kMStages], A.ctl, A.timeout_ns, 84);
      if (__syncthreads_or(bad)) {
        for (int j = i + 1; j < issued; ++j) mbar_wait(&sm.kfull[stq[j % kMStages]], paq[j % kMStages], A.ctl,
                                                       A.timeout_ns, 85);
        return false;
      }
      const float* kb = sm.kb[st];
      float av[kOwnPerLane];
#pragma unroll
      for (int j = 0; j < kOwnPerLane; ++j) av[j] = sm.ab[st][lane + 32 * j];
      // sub-block qi holds this warp's columns 4 qi .. 4 qi + 3
      const int qi = i % nq;
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) {
        if (qi != qq) continue;
#pragma unroll
        for (int c4 = 0; c4 < kSubCols / kWarps; ++c4) {
          const int c = warp + kWarps * c4;  // column within the sub-block
          if (c < cur.ncols) {
            float sacc = 0.f;
#pragma unroll
            for (int j = 0; j < kOwnPerLane; ++j) sacc = fmaf(kb[c * kBlockPts + lane + 32 * j], av[j], sacc);
            acc[4 * qq + c4] += sacc;
          }
        }
      }
      __syncthreads();
    }
    // column sums across lanes: column (w + 8 (4 qq + c4)) of the block = 32 qq + w + 8 c4
#pragma unroll
    for (int i = 0; i < kColsPerWarp; ++i) {
      float v = acc[i];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0) sm.colsum[32 * (i >> 2) + warp + kWarps * (i & 3)] = v;
    }
    __syncthreads();
    float tot[1] = {threadIdx.x < kBlockPts ? sm.colsum[threadIdx.x] : 0.f};
    if (split_complete<1>(sm, g, cbk, sl, round, A.part, A.cnt_c, tot)) fin0(cbk, tot);
  }
  return true;
}

__global__ void __launch_bounds__(kThreads, 2) softassign_mat_kernel(const MatArgs A) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  MatSmem& sm = *reinterpret_cast<MatSmem*>(smem_raw);
  __shared__ float s_pose[12];
  __shared__ df s_red[kThreads];
  __shared__ df s_tot[kSaNV];
  __shared__ float s_hdr[12];
  __shared__ float s_S[9], s_xcp[3], s_yd[3], s_xc[3], s_yc[3];
  __shared__ HornState<float> horn;

  const int tid = threadIdx.x;
  const unsigned G = gridDim.x;
  if (tid == 0) {
    for (int s = 0; s < kMStages; ++s) mbar_init(&sm.kfull[s], 1);
    for (int s = 0; s < 2; ++s) mbar_init(&sm.full[s], 1);
    mbar_init_fence();
    for (int k = 0; k < 3; ++k) {
      s_hdr[k] = A.hdr->oX[k];
      s_hdr[3 + k] = A.hdr->oY[k];
      s_hdr[6 + k] = A.hdr->ymean[k];
    }
    float R[9], t[3], tc[3];
    for (int k = 0; k < 9; ++k) R[k] = A.dRt[k];
    for (int k = 0; k < 3; ++k) t[k] = A.dRt[9 + k];
    pose_to_centred(R, t, &s_hdr[0], &s_hdr[3], tc);
    for (int k = 0; k < 9; ++k) s_pose[k] = R[k];
    for (int k = 0; k < 3; ++k) s_pose[9 + k] = tc[k];
    horn.reset();
  }
  __syncthreads();

  KRing rg{{0u, 0u, 0u}, 0};
  unsigned wuses[2] = {0u, 0u};
  unsigned epoch = 0, rr = 0, rc = 0;  // sweeps completed per geometry (split counters)
  float T = A.T0;
  int step = 0;
  bool ok = true;
  const float* wb1[1] = {A.b};
  const float* wb5[5] = {A.w5, A.w5 + A.Mp, A.w5 + 2 * (size_t)A.Mp, A.w5 + 3 * (size_t)A.Mp,
                         A.w5 + 4 * (size_t)A.Mp};
  auto barrier = [&](int where) {
    if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, where)) return false;
    // K, weights and a written before the barrier are read by the copy engine next
    if (tid == 0) asm volatile("fence.proxy.async.global;" ::: "memory");
    return true;
  };
  for (int Titer = 0; Titer < A.JMAX && ok; ++Titer) {
    const float kk = kLog2e / T;
    const float nk = -kk;
    const float c0 = fmaf(A.alpha, kk, -0.5f * log2f(T));
    for (int iter0 = 0; iter0 < A.I0 && ok; ++iter0, ++step) {
      float R[9], tc[3];
#pragma unroll
      for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
      __syncthreads();
      ok = pass_write(sm, A, rr++, R, tc, nk, c0, wuses) && barrier(86);
      for (int k = 0; k < A.I1 && ok; ++k) {
        if (k >= 1) {
          ok = pass_rows<1>(sm, rg, A, rr++, wb1, MatRowFin{A.a, A.s, A.rs, A.N, false}) && barrier(87);
          if (!ok) break;
        }
        const MatColFin cf{A.b, A.u, A.cs, A.w5, A.M, A.Mp, k == 0, k == A.I1 - 1, A.cols,
                           {s_hdr[6], s_hdr[7], s_hdr[8]}, reinterpret_cast<df*>(sm.raw),
                           A.rec + (size_t)A.gr.nblk * 32};
        ok = pass_cols(sm, rg, A, rc++, cf) && barrier(88);
      }
      if (!ok) break;
      const FinalFin ff{A.rows, A.a, A.w_out, A.N, reinterpret_cast<df*>(sm.raw), A.rec};
      ok = pass_rows<5>(sm, rg, A, rr++, wb5, ff) && barrier(89);
      if (!ok) break;
      reduce_block_partials<32>(A.rec, A.gr.nblk + A.gc.nblk, s_red, s_tot);
      if (tid < 12)
        sa_moments_to_S(tid, s_tot, &s_hdr[0], &s_hdr[3], &s_hdr[6], s_S, s_xcp, s_yd, s_xc, s_yc);
      __syncthreads();
      if (tid == 0) {
        float S[9], Xcp[3], Yd[3];
        for (int k = 0; k < 9; ++k) S[k] = s_S[k];
        for (int i = 0; i < 3; ++i) {
          Xcp[i] = s_xcp[i];
          Yd[i] = s_yd[i];
        }
        float q[4], gap = 0.f, lmax = 0.f, Rn[9], tn[3];
        horn_quaternion<float>(S, horn, q, &gap, &lmax);
        quat_to_pose<float>(q, Xcp, Yd, Rn, tn);
        for (int k = 0; k < 9; ++k) s_pose[k] = Rn[k];
        for (int k = 0; k < 3; ++k) s_pose[9 + k] = tn[k];
        if (blockIdx.x == 0) {
          if (A.trace && step < A.trace_cap) {
            double* rec = A.trace + (size_t)step * 32;
            float to[3];
            pose_from_centred(Rn, tn, &s_hdr[0], &s_hdr[3], to);
            rec[0] = step;
            rec[1] = T;
            rec[2] = df_dbl(s_tot[0]);
            for (int i = 0; i < 3; ++i) {
              rec[3 + i] = s_xc[i];
              rec[6 + i] = s_yc[i];
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
    }
    T = T * A.TFACTOR;  // FP32, src/softassign.cu:820
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
  }
}

// ------------------------------------------------------------------ host side
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

// Slices in whole quanta (sub-block columns or row blocks), chosen by a cost
// model of one pass: waves of units over the grid, each unit moving its share
// of K at the per-block share of HBM bandwidth plus a fixed start-up time
// (first copy latency, completion).
SweepGeom mat_geom(int n_own, int n_stream, int quantum, int grid, double bytes_per_quantum_per_block) {
  SweepGeom g;
  g.n_own = n_own;
  g.n_stream = n_stream;
  g.nblk = (n_own + kBlockPts - 1) / kBlockPts;
  const int qn = (n_stream + quantum - 1) / quantum;  // streamed quanta
  const double per_block_bw = 7.0e12 / (double)grid;   // bytes/s
  const double startup = 3.0e-6;
  double best = 1e300;
  int bestS = 1;
  for (int S = 1; S <= qn && S <= 4096; ++S) {
    const int per = (qn + S - 1) / S;
    const int s_eff = (qn + per - 1) / per;
    if (s_eff != S) continue;
    const long units = (long)g.nblk * S;
    const long waves = (units + grid - 1) / grid;
    const double cost = (double)waves * ((double)per * bytes_per_quantum_per_block / per_block_bw + startup);
    if (cost < best) {
      best = cost;
      bestS = S;
    }
  }
  const int per = (qn + bestS - 1) / bestS;
  g.slice_len = per * quantum;
  g.slices = (n_stream + g.slice_len - 1) / g.slice_len;
  g.units = g.nblk * g.slices;
  return g;
}

struct MatPlan {
  int grid;
  SweepGeom gr, gc;
  size_t smem;
};

MatPlan plan_mat(int N, int M, int device) {
  MatPlan P;
  P.smem = sizeof(MatSmem);
  const int limit = persistent_grid_limit(device, (const void*)softassign_mat_kernel, P.smem);
  // a row-pass quantum is one 32-column sub-block (16 KiB); a column-pass
  // quantum is one row block (128 rows x 128 columns, 64 KiB)
  P.gr = mat_geom(N, M, kSubCols, limit, (double)kSubFloats * 4.0);
  const int nblk_r = P.gr.nblk;
  P.gc = mat_geom(M, nblk_r, 1, limit, (double)kBlockPts * kBlockPts * 4.0);
  const int mu = P.gr.units > P.gc.units ? P.gr.units : P.gc.units;
  P.grid = mu < limit ? mu : limit;
  return P;
}

struct MatCarved {
  Ctl* ctl;
  unsigned *cnt_r, *cnt_c;
  CenterHdr* hdr;
  float4 *rows, *cols;
  float* K;
  float *a, *s, *rs, *b, *u, *cs, *w5;
  float* part;
  df* rec;
  int Mp;
};

MatCarved carve_mat(void* base, const MatPlan& P, int N, int M, size_t* total, size_t* zero_bytes) {
  Carve c(base);
  MatCarved w;
  const size_t rows_pad = (size_t)P.gr.nblk * kBlockPts;
  w.Mp = (M + 3) & ~3;
  w.ctl = c.take<Ctl>(1);
  w.cnt_r = c.take<unsigned>((size_t)P.gr.nblk);
  w.cnt_c = c.take<unsigned>((size_t)P.gc.nblk);
  w.a = c.take<float>(rows_pad);  // zero beyond N (multiplies the padded rows of K)
  if (zero_bytes) *zero_bytes = c.off;
  w.hdr = c.take<CenterHdr>(1);
  w.rows = c.take<float4>((size_t)N);
  w.cols = c.take<float4>((size_t)M);
  w.s = c.take<float>(rows_pad);
  w.rs = c.take<float>(rows_pad);
  w.b = c.take<float>((size_t)w.Mp);
  w.u = c.take<float>((size_t)w.Mp);
  w.cs = c.take<float>((size_t)w.Mp);
  w.w5 = c.take<float>((size_t)5 * w.Mp);
  const size_t pr = (size_t)P.gr.units * 5 * kBlockPts, pc = (size_t)P.gc.units * kBlockPts;
  w.part = c.take<float>(pr > pc ? pr : pc);
  w.rec = c.take<df>((size_t)(P.gr.nblk + P.gc.nblk) * 32);
  w.K = c.take<float>(rows_pad * (size_t)M);
  if (total) *total = c.off;
  return w;
}

}  // namespace

size_t softassign_mat_ws_need(int N, int M, int device) {
  const MatPlan P = plan_mat(N, M, device);
  size_t total = 0;
  carve_mat(nullptr, P, N, M, &total, nullptr);
  return total;
}

int enqueue_softassign_mat(const SoftassignLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  const MatPlan P = plan_mat(L.N, L.M, device);
  size_t total = 0, zero_bytes = 0;
  MatCarved w = carve_mat(ws, P, L.N, L.M, &total, &zero_bytes);
  if (total > ws_bytes) return (int)cudaErrorInvalidValue;
  if (grid_used) *grid_used = P.grid;
  // control block, split counters and a (padding rows must be zero) start at zero
  e = cudaMemsetAsync(ws, 0, zero_bytes, st);
  if (e != cudaSuccess) return (int)e;
  prep_center_kernel<<<1, 1024, 0, st>>>(L.dX, L.N, L.dY, L.M, w.hdr);
  const int pb = 256, pg_x = (L.N + pb - 1) / pb, pg_y = (L.M + pb - 1) / pb;
  prep_pack_kernel<<<pg_x < 1024 ? pg_x : 1024, pb, 0, st>>>(L.dX, L.N, w.hdr, 0, 0.f, w.rows);
  prep_pack_kernel<<<pg_y < 1024 ? pg_y : 1024, pb, 0, st>>>(L.dY, L.M, w.hdr, 1, 0.f, w.cols);
  if (L.s_io)
    e = cudaMemcpyAsync(w.s, L.s_io, sizeof(float) * (size_t)L.N, cudaMemcpyDeviceToDevice, st);
  else
    fill_kernel<<<pg_x < 1024 ? pg_x : 1024, pb, 0, st>>>(w.s, L.N, L.moutlier);
  if (e == cudaSuccess && L.u_io)
    e = cudaMemcpyAsync(w.u, L.u_io, sizeof(float) * (size_t)L.M, cudaMemcpyDeviceToDevice, st);
  else if (e == cudaSuccess)
    fill_kernel<<<pg_y < 1024 ? pg_y : 1024, pb, 0, st>>>(w.u, L.M, L.moutlier);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (L.JMAX <= 0 || L.I0 <= 0) return 0;
  MatArgs A;
  A.rows = w.rows;
  A.cols = w.cols;
  A.K = w.K;
  A.a = w.a;
  A.s = w.s;
  A.rs = w.rs;
  A.b = w.b;
  A.u = w.u;
  A.cs = w.cs;
  A.w5 = w.w5;
  A.w_out = L.w_out;
  A.N = L.N;
  A.M = L.M;
  A.Mp = w.Mp;
  A.gr = P.gr;
  A.gc = P.gc;
  A.JMAX = L.JMAX;
  A.I0 = L.I0;
  A.I1 = L.I1;
  A.alpha = L.alpha;
  A.T0 = L.T_0;
  A.TFACTOR = L.TFACTOR;
  A.hdr = w.hdr;
  A.dRt = L.dRt;
  A.part = w.part;
  A.cnt_r = w.cnt_r;
  A.cnt_c = w.cnt_c;
  A.rec = w.rec;
  A.ctl = w.ctl;
  A.trace = L.trace;
  A.trace_cap = L.trace_cap;
  A.d_status = L.d_status;
  A.timeout_ns = L.timeout_ns;
  void* args[] = {(void*)&A};
  e = cudaLaunchCooperativeKernel((const void*)softassign_mat_kernel, dim3(P.grid), dim3(kThreads), args, P.smem,
                                  st);
  if (e != cudaSuccess) return (int)e;
  // outputs of the schedule's last pose update
  if (L.s_io) e = cudaMemcpyAsync(L.s_io, w.s, sizeof(float) * (size_t)L.N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && L.u_io)
    e = cudaMemcpyAsync(L.u_io, w.u, sizeof(float) * (size_t)L.M, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && L.rs_out)
    e = cudaMemcpyAsync(L.rs_out, w.rs, sizeof(float) * (size_t)L.N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && L.cs_out)
    e = cudaMemcpyAsync(L.cs_out, w.cs, sizeof(float) * (size_t)L.M, cudaMemcpyDeviceToDevice, st);
  return (int)e;
}

}  // namespace cesa
