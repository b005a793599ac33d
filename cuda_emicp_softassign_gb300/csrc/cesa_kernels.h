// Host-visible launch interface of the registration kernels (internal to
// libcesa.so; the public C ABI is include/cesa.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

struct cesa_params;

namespace cesa {

// Argument checks of the C ABI (cesa_api.cu), shared by every entry point:
// CESA_OK or CESA_ERR_INVALID_ARGUMENT.
int check_points(const float* X, int N, const float* Y, int M);
int check_emicp_params(const cesa_params* p);
// Sigma steps of the EM-ICP schedule (stepped in FP32), or -1 if it never ends.
long emicp_steps(float sigma_p2, float sigma_inf, float sigma_factor);
// Limit of the device-side waits in ns (p->timeout_ms, 0 selects 10 s).
uint64_t timeout_ns_of(const cesa_params* p);
// The lock every entry point holds while it plans and enqueues.
std::mutex& api_mutex();
// Records that the last call on (dev, st) ran on the no-allocation scratch,
// whose control block cesa_stream_status then reads. Call with api_mutex held.
void note_noalloc_call(int dev, cudaStream_t st, void* scratch);

struct SweepGeomH {
  int n_own, n_stream, nblk, slices, slice_len, units;
};

// Centering header computed on the device by prep_center_kernel.
struct CenterHdr {
  float oX[4];     // FP32 offset subtracted from X (mean of X rounded to float)
  float oY[4];     // same for Y
  float xmean[4];  // mean of the centred X' (used by EM-ICP rows with C_r <= 1e-6)
  float ymean[4];
};

// Pose I/O block: R (9, row-major) and t (3) in the caller's frame.
struct PoseIO {
  float R[9];
  float t[3];
};

struct EmicpLaunch {
  const float* dX;  // SoA, N
  const float* dY;  // SoA, M
  int N, M;
  float sigma_p2, sigma_factor, d_02;
  int nsteps;
  float* dRt;        // PoseIO in/out (device)
  float* row_out;    // optional [M][5]
  double* trace;     // optional device trace [cap][32]
  int trace_cap;
  int* d_status;     // optional device status mirror
  unsigned long long* timeline;  // optional device phase timeline (block 0)
  int timeline_cap;
  uint64_t timeout_ns;
  float* tape;       // optional [nsteps][kEmTape] step records for the adjoint
  float* row_tape;   // optional [nsteps][M][5] per-row (C, lambda, u), centred frame
};

// EM-ICP tape record per step (floats): [0..8] R in, [9..11] t' in (centred
// frame), [12] sigma_p2, [16..47] the 16 moments as (hi, lo), [48..63] Horn
// eigenbasis V (row-major, columns are eigenvectors), [64..67] q.
constexpr int kEmTape = 80;

struct SoftassignLaunch {
  const float* dX;  // SoA, N (rows of the match matrix)
  const float* dY;  // SoA, M (columns)
  int N, M;
  int JMAX, I0, I1;
  float alpha, T_0, TFACTOR, moutlier;
  int form;          // CESA_SINKHORN_MATRIX_FREE / _MATERIALISED (resolved)
  float* dRt;        // PoseIO in/out (device)
  float* s_io;       // optional slack column in/out [N] (else initialised to moutlier)
  float* u_io;       // optional slack row in/out [M]
  float* rs_out;     // optional [N]
  float* cs_out;     // optional [M]
  float* w_out;      // optional [N]
  double* trace;
  int trace_cap;
  int* d_status;
  unsigned long long* timeline;
  int timeline_cap;
  uint64_t timeout_ns;
  // optional tape of the matrix-free form, per pose update n:
  //   tape_pose [n][kSaTape]: input pose (centred), sumM, centres, S, q, eigenbasis
  //   tape_s [n][N], tape_u [n][M]: the input slack
  //   tape_rows [n][I1][4][N]: per row pass k: a^(k+1), s^(k+1), rs^k, r^k
  //   tape_cols [n][I1][4][M]: per column pass k: b^(k+1), u^(k+1), cs^k, c^k
  //   tape_fin [n][5][N]: the final sweep's row sums K b, K (b (cs - 1)), K (b cs (y' - Yhat))
  float* tape_pose;
  float* tape_s;
  float* tape_u;
  float* tape_rows;
  float* tape_cols;
  float* tape_fin;
};
// Softassign tape record of one pose update (floats):
//   0-11 input pose (R, t', centred)  12-13 sumM (hi, lo)  14-16 Xc  17-19 Yc (caller frame)
//   20-22 Xc - oX  23-25 Yc - oY  26-34 S  35-38 q  39-54 Horn eigenbasis V[4][4]
constexpr int kSaTape = 64;

// One pair of a batched launch (device pointers).
constexpr int kMaxBatchPairs = 1024;
struct BatchLaunchPair {
  int algo;  // 0 EM-ICP, 1 Softassign
  int N, M;
  const float* dX;  // SoA, N
  const float* dY;  // SoA, M
  float* dRt;       // PoseIO in/out (device)
  int nsteps;       // EM-ICP sigma steps
  float sigma_p2, sigma_factor, d_02;
  int JMAX, I0, I1;  // Softassign
  float alpha, T_0, TFACTOR, moutlier;
};

// Sinkhorn forms of SoftassignLaunch.form (the CESA_SINKHORN_* values).
constexpr int kFormMatrixFree = 1;
constexpr int kFormMaterialised = 2;
constexpr int kFormBanded = 3;  // matrix-free arithmetic, one thread-block cluster per band of rows

// Device workspace carved from one allocation (see api.cu).
struct Workspace {
  void* base = nullptr;
  size_t bytes = 0;
};

size_t emicp_workspace_bytes(int N, int M, int grid, const SweepGeomH& g);
size_t softassign_workspace_bytes(int N, int M, int grid, const SweepGeomH& gr, const SweepGeomH& gc,
                                  int form);

// Plans the persistent grid and the unit decomposition.
int persistent_grid_limit(int device, const void* kernel, size_t smem);
SweepGeomH plan_sweep(int n_own, int n_stream, int grid_limit);

// Enqueue a full registration; returns cudaError_t as int.
int enqueue_emicp(const EmicpLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used);
int enqueue_softassign(const SoftassignLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st,
                       int* grid_used);
size_t emicp_ws_need(int N, int M, int device);
size_t softassign_ws_need(int N, int M, int form, int device);
size_t softassign_mat_ws_need(int N, int M, int device);
int enqueue_softassign_mat(const SoftassignLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used);
// Banded form: fits when M <= 2048 and all nb = ceil(N / 64) clusters can be
// resident at once; preferred (AUTO without a tuned decision) when it also
// occupies at least half of the SMs and nb <= 48.
bool softassign_band_fits(int N, int M, int device);
bool softassign_band_preferred(int N, int M, int device);
size_t softassign_band_ws_need(int N, int M, int device);
int enqueue_softassign_band(const SoftassignLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used);

// Batched registration: all pairs in one persistent launch.
size_t batch_ws_need(const BatchLaunchPair* pairs, int npairs, int device);
int enqueue_batch(const BatchLaunchPair* pairs, int npairs, int* d_status, uint64_t timeout_ns, void* ws,
                  size_t ws_bytes, cudaStream_t st, int* grid_used, int* rounds_out);

// EM-ICP adjoint over a recorded forward (tape).
struct EmicpAdjointLaunch {
  const float4* rows;  // Y' centred (M), as packed by the forward
  const float4* cols;  // X' centred (N)
  const CenterHdr* hdr;
  int N, M, nsteps;
  const float* tape;      // [nsteps][kEmTape]
  const float* row_tape;  // [nsteps][M][5]
  const float* g_out;     // device [12]: dL/dR (9), dL/dt (3) of the final pose, caller frame
  float* gX;              // device SoA [3N] (written)
  float* gY;              // device SoA [3M] (written)
  float* g_in;            // device [12]: dL/dR0, dL/dt0 of the initial pose, caller frame
  int* d_status;
  uint64_t timeout_ns;
  int layout;             // CESA_LAYOUT_*
};
size_t emicp_adjoint_ws_need(int N, int M, int device, int layout);
int enqueue_emicp_adjoint(const EmicpAdjointLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st);
// The forward workspace's packed clouds and centring header (for the tape).
void emicp_ws_views(void* ws, int N, int M, int device, CenterHdr** hdr, float4** rows, float4** cols);

void softassign_ws_views(void* ws, int N, int M, int device, CenterHdr** hdr, float4** rows, float4** cols);

// Softassign adjoint over a recorded tape (device pointers). One update's
// backward is the same launch sequence for every update: a device counter
// selects the update's tape slices from a table, which a first kernel copies
// into fixed workspace buffers, and the last kernel steps the counter. The
// sequence can therefore be captured once as a CUDA graph and replayed.
struct SaUpdate {
  const float* rec;   // [kSaTape]
  const float* s0;    // [N]
  const float* u0;    // [M]
  const float* rows;  // [I1][4][N]
  const float* cols;  // [I1][4][M]
  const float* fin;   // [5][N]
  float T;
  int pad;
};
struct SoftassignBackward {
  const float4* X;    // X' centred (N), as packed by the forward
  const float4* Y;    // Y' centred (M)
  const CenterHdr* hdr;
  int N, M, I1;
  long nsteps;
  float alpha;
  const float* g_out; // [12] dL/dR, dL/dt of the final pose (caller frame)
  float* gX;          // SoA [3N] (written by finish)
  float* gY;          // SoA [3M]
  float* g_in;        // [12] dL/d(R, t) of the initial pose
};
size_t softassign_bwd_ws_need(int N, int M, int I1, long nsteps);
int softassign_bwd_prepare(const SoftassignBackward& B, const SaUpdate* host_tab, void* ws, size_t ws_bytes,
                           cudaStream_t st);
int softassign_bwd_update(const SoftassignBackward& B, void* ws, size_t ws_bytes, cudaStream_t st);
int softassign_bwd_finish(const SoftassignBackward& B, void* ws, size_t ws_bytes, cudaStream_t st);
// The whole backward as one persistent cooperative launch (the updates in
// reverse, the stages separated by grid barriers with a time limit); writes
// dL/dX, dL/dY, dL/d(R0, t0) and the device status (d_status, nullable, and
// the workspace's control block). cudaErrorCooperativeLaunchTooLarge when it
// cannot be launched on this device.
int softassign_bwd_persistent(const SoftassignBackward& B, const SaUpdate* host_tab, void* ws, size_t ws_bytes,
                              cudaStream_t st, int* d_status, uint64_t timeout_ns);

// ICP (exhaustive nearest neighbours): maxIteration iterations in one launch.
struct IcpLaunch {
  const float* dX;  // SoA, N (searched)
  const float* dY;  // SoA, M (moved)
  int N, M, iters;
  float* dRt;       // PoseIO in/out (device)
  int* nn_out;      // optional [M]: the last iteration's matches
  int search;       // CESA_ICP_SEARCH_*
  double* trace;
  int trace_cap;
  int* d_status;
  uint64_t timeout_ns;
};
size_t icp_ws_need(int N, int M, int device, int search);
int enqueue_icp(const IcpLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used);

// Control-block status of the last launch that used workspace ws.
int read_ws_status(void* ws, cudaStream_t st, int* status, int* steps, int* tl_written = nullptr);

}  // namespace cesa
