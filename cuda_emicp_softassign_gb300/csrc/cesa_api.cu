// C ABI of libcesa.so (declared in include/cesa.h).
//
// Host-pointer entry points keep the reference's calling convention: they
// return only after R,t have been written back. Unlike the reference
// (src/emicp.cu:713, src/softassign.cu:885), they never reset the device.
// Device memory (point copies, workspace, trace) is cached per
// (device, stream) and reused by later calls with the same or smaller sizes.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/cesa.h"
#include "cesa_kernels.h"
#include "cesa_pose.h"

namespace cesa {
namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t need) {
    if (need <= bytes && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    bytes = need;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

// The Softassign backward's per-update launches, captured as a CUDA graph for
// one workspace layout and replayed once per update (on a stream of its own,
// ordered after and before the caller's stream by events).
struct SaBwdGraph {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  void* ws = nullptr;
  size_t bytes = 0;
  int N = 0, M = 0, I1 = 0;
  float alpha = 0.f;
  void release() {
    if (stream) cudaStreamSynchronize(stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (stream) cudaStreamDestroy(stream);
    *this = SaBwdGraph{};
  }
};

struct StreamCtx {
  DevBuf ws;     // kernel workspace (control block first)
  DevBuf io;     // point copies + pose + outputs for host-pointer calls
  DevBuf trace;  // device trace records
  DevBuf tl;     // device phase timeline
  SaBwdGraph sa_bwd;
  int last_trace_steps = 0;
  int last_kind = 0;  // 1 emicp, 2 softassign
};

std::mutex g_mu;
std::map<std::pair<int, cudaStream_t>, StreamCtx> g_ctx;
std::map<int, cudaStream_t> g_own_stream;

// Streams whose last call was cesa_emicp_device_noalloc, with the control
// block of its fixed scratch. A fixed table, so that recording a no-allocation
// call allocates nothing, not even host memory; when it is full the oldest
// record is replaced. Guarded by g_mu.
struct NoallocRec {
  int dev = -1;
  cudaStream_t st = nullptr;
  void* ctl = nullptr;
};
constexpr int kNoallocRecs = 64;
NoallocRec g_noalloc_rec[kNoallocRecs];
int g_noalloc_next = 0;

NoallocRec* noalloc_rec(int dev, cudaStream_t st) {
  for (auto& r : g_noalloc_rec)
    if (r.ctl && r.dev == dev && r.st == st) return &r;
  return nullptr;
}

// The context of a call that enqueues work on (dev, st): from here on the
// stream's status is that of this call's workspace.
StreamCtx& ctx_for(int dev, cudaStream_t st) {
  if (NoallocRec* r = noalloc_rec(dev, st)) *r = NoallocRec{};
  return g_ctx[std::make_pair(dev, st)];
}

// Largest N x M whose Softassign backward runs as one persistent launch.
constexpr double kSaBwdPersistentMaxElems = 16.0e6;

int map_cuda(cudaError_t e) {
  if (e == cudaSuccess) return CESA_OK;
  if (e == cudaErrorMemoryAllocation) return CESA_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return CESA_ERR_NO_DEVICE;
  if (e == cudaErrorCooperativeLaunchTooLarge) return CESA_ERR_UNSUPPORTED;
  return CESA_ERR_CUDA;
}

}  // namespace

// Argument checks and schedule length shared by the entry points of this
// file and cesa_noalloc.cu (declared in cesa_kernels.h).
uint64_t timeout_ns_of(const cesa_params* p) {
  const int ms = (p && p->timeout_ms > 0) ? p->timeout_ms : 10000;
  return (uint64_t)ms * 1000000ull;
}

// Number of sigma steps of src/emicp.cu:443,668 (FP32 loop), or -1 if it
// would never end.
long emicp_steps(float sigma_p2, float sigma_inf, float sigma_factor) {
  long n = 0;
  float s = sigma_p2;
  while (s > sigma_inf) {
    ++n;
    s *= sigma_factor;
    if (n > 100000000L) return -1;
  }
  return n;
}

int check_points(const float* X, int N, const float* Y, int M) {
  if (!X || !Y || N < 1 || M < 1) return CESA_ERR_INVALID_ARGUMENT;
  if ((long)N * 16 > 0x7fffffffL || (long)M * 16 > 0x7fffffffL) return CESA_ERR_INVALID_ARGUMENT;
  return CESA_OK;
}

int check_emicp_params(const cesa_params* p) {
  if (!p) return CESA_ERR_INVALID_ARGUMENT;
  if (!(p->sigma_p2 > 0.f) || !(p->sigma_inf > 0.f) || !(p->sigma_factor > 0.f) ||
      !(p->d_02 >= 0.f) || !isfinite(p->sigma_p2))
    return CESA_ERR_INVALID_ARGUMENT;
  if (p->sigma_p2 > p->sigma_inf && !(p->sigma_factor < 1.f)) return CESA_ERR_INVALID_ARGUMENT;
  return CESA_OK;
}

namespace {

int check_sa_params(const cesa_params* p) {
  if (!p) return CESA_ERR_INVALID_ARGUMENT;
  if (p->JMAX < 0 || p->I0 < 0 || p->I1 < 1) return CESA_ERR_INVALID_ARGUMENT;
  if (!(p->T_0 > 0.f) || !(p->TFACTOR > 0.f) || !isfinite(p->alpha) || !(p->moutlier >= 0.f))
    return CESA_ERR_INVALID_ARGUMENT;
  if ((long)p->JMAX * (long)p->I0 > 100000000L) return CESA_ERR_INVALID_ARGUMENT;
  return CESA_OK;
}

int check_icp_params(const cesa_params* p) {
  if (!p) return CESA_ERR_INVALID_ARGUMENT;
  if (p->maxIteration < 0 || p->maxIteration > 100000000) return CESA_ERR_INVALID_ARGUMENT;
  if (p->icp_search < CESA_ICP_SEARCH_AUTO || p->icp_search > CESA_ICP_SEARCH_GRID) return CESA_ERR_INVALID_ARGUMENT;
  return CESA_OK;
}

int select_device(const cesa_params* p, int* dev) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return CESA_ERR_NO_DEVICE;
  if (p && p->device >= 0) {
    if (p->device >= n) return CESA_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(p->device) != cudaSuccess) return CESA_ERR_CUDA;
  }
  if (cudaGetDevice(dev) != cudaSuccess) return CESA_ERR_CUDA;
  return CESA_OK;
}

cudaStream_t own_stream(int dev) {
  auto it = g_own_stream.find(dev);
  if (it != g_own_stream.end()) return it->second;
  cudaStream_t s = nullptr;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  g_own_stream[dev] = s;
  return s;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static_assert(kFormMatrixFree == CESA_SINKHORN_MATRIX_FREE && kFormMaterialised == CESA_SINKHORN_MATERIALISED &&
                  kFormBanded == CESA_SINKHORN_BANDED,
              "Sinkhorn form values");

// Sinkhorn form chosen per size by the tuner (cesa_tune_sinkhorn): measured
// decisions per device and half-octave size bucket of (N, M).
struct TuneKey {
  int dev, bn, bm;
  bool operator<(const TuneKey& o) const {
    return dev != o.dev ? dev < o.dev : (bn != o.bn ? bn < o.bn : bm < o.bm);
  }
};
std::map<TuneKey, int> g_tuned;  // guarded by g_mu

int size_bucket(int n) { return (int)floor(2.0 * log2((double)(n > 1 ? n : 1))); }

// The materialised form needs its N x M matrix: never chosen when that would
// take more than half of the device's free memory.
bool materialised_fits(int N, int M) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
  const double k_bytes = (double)((N + 127) / 128 * 128) * (double)M * 4.0;
  return k_bytes < 0.5 * (double)free_b;
}

// Form for a request. BANDED falls back to the matrix-free form where the
// clouds do not fit it. AUTO takes the tuner's decision for the size bucket;
// without one, the banded form where it fits and fills the GPU, else the
// matrix-free form (the materialised form streams 28 bytes per element per
// update and has not been faster on GB300).
int resolve_form(int requested, int N, int M, int dev) {
  if (requested == CESA_SINKHORN_MATRIX_FREE) return kFormMatrixFree;
  if (requested == CESA_SINKHORN_MATERIALISED) return kFormMaterialised;
  if (requested == CESA_SINKHORN_BANDED) return softassign_band_fits(N, M, dev) ? kFormBanded : kFormMatrixFree;
  auto it = g_tuned.find(TuneKey{dev, size_bucket(N), size_bucket(M)});
  if (it != g_tuned.end() && (it->second != kFormMaterialised || materialised_fits(N, M)) &&
      (it->second != kFormBanded || softassign_band_fits(N, M, dev)))
    return it->second;
  return softassign_band_preferred(N, M, dev) ? kFormBanded : kFormMatrixFree;
}

// Shared body of the two host-pointer entry points.
int run_host(int kind, const float* X, int N, const float* Y, int M, float R[9], float t[3],
             const cesa_params* p, cesa_report* rep) {
  int rc = check_points(X, N, Y, M);
  if (rc) return rc;
  if (!R || !t) return CESA_ERR_INVALID_ARGUMENT;
  rc = kind == 1 ? check_emicp_params(p) : kind == 2 ? check_sa_params(p) : check_icp_params(p);
  if (rc) return rc;
  long nsteps = kind == 1   ? emicp_steps(p->sigma_p2, p->sigma_inf, p->sigma_factor)
                : kind == 2 ? (long)p->JMAX * (long)p->I0
                            : (long)p->maxIteration;
  if (nsteps < 0) return CESA_ERR_INVALID_ARGUMENT;
  int dev = 0;
  rc = select_device(p, &dev);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t st = own_stream(dev);
  StreamCtx& C = ctx_for(dev, st);
  const size_t bx = align256(sizeof(float) * 3 * (size_t)N);
  const size_t by = align256(sizeof(float) * 3 * (size_t)M);
  cudaError_t e = C.io.ensure(bx + by + 256);
  if (e != cudaSuccess) return map_cuda(e);
  float* dX = static_cast<float*>(C.io.p);
  float* dY = reinterpret_cast<float*>(static_cast<char*>(C.io.p) + bx);
  float* dRt = reinterpret_cast<float*>(static_cast<char*>(C.io.p) + bx + by);
  const int form = kind == 2 ? resolve_form(p->sinkhorn_form, N, M, dev) : 0;
  const size_t need = kind == 1   ? emicp_ws_need(N, M, dev)
                      : kind == 2 ? softassign_ws_need(N, M, form, dev)
                                  : icp_ws_need(N, M, dev, p->icp_search);
  e = C.ws.ensure(need);
  if (e != cudaSuccess) return map_cuda(e);
  const int cap = (rep && rep->trace && rep->trace_capacity > 0) ? rep->trace_capacity : 0;
  double* dtrace = nullptr;
  if (cap > 0) {
    e = C.trace.ensure(sizeof(double) * 32 * (size_t)cap);
    if (e != cudaSuccess) return map_cuda(e);
    dtrace = static_cast<double*>(C.trace.p);
  }
  const int tl_cap = (rep && rep->timeline && rep->timeline_capacity > 0) ? rep->timeline_capacity : 0;
  unsigned long long* dtl = nullptr;
  if (tl_cap > 0) {
    e = C.tl.ensure(sizeof(unsigned long long) * (size_t)tl_cap);
    if (e == cudaSuccess) e = cudaMemsetAsync(C.tl.p, 0, sizeof(unsigned long long) * (size_t)tl_cap, st);
    if (e != cudaSuccess) return map_cuda(e);
    dtl = static_cast<unsigned long long*>(C.tl.p);
  }
  float hRt[12];
  memcpy(hRt, R, sizeof(float) * 9);
  memcpy(hRt + 9, t, sizeof(float) * 3);
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  e = cudaMemcpyAsync(dX, X, sizeof(float) * 3 * (size_t)N, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dY, Y, sizeof(float) * 3 * (size_t)M, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dRt, hRt, sizeof(hRt), cudaMemcpyHostToDevice, st);
  int grid = 0;
  int kerr = 0;
  if (e == cudaSuccess) {
    cudaEventRecord(ev0, st);
    if (kind == 1) {
      EmicpLaunch L{};
      L.dX = dX;
      L.dY = dY;
      L.N = N;
      L.M = M;
      L.sigma_p2 = p->sigma_p2;
      L.sigma_factor = p->sigma_factor;
      L.d_02 = p->d_02;
      L.nsteps = (int)nsteps;
      L.dRt = dRt;
      L.trace = dtrace;
      L.trace_cap = cap;
      L.timeline = dtl;
      L.timeline_cap = tl_cap;
      L.timeout_ns = timeout_ns_of(p);
      kerr = enqueue_emicp(L, C.ws.p, C.ws.bytes, st, &grid);
    } else if (kind == 3) {
      IcpLaunch L{};
      L.dX = dX;
      L.dY = dY;
      L.N = N;
      L.M = M;
      L.iters = (int)nsteps;
      L.search = p->icp_search;
      L.dRt = dRt;
      L.trace = dtrace;
      L.trace_cap = cap;
      L.timeout_ns = timeout_ns_of(p);
      kerr = enqueue_icp(L, C.ws.p, C.ws.bytes, st, &grid);
    } else {
      SoftassignLaunch L{};
      L.dX = dX;
      L.dY = dY;
      L.N = N;
      L.M = M;
      L.JMAX = p->JMAX;
      L.I0 = p->I0;
      L.I1 = p->I1;
      L.alpha = p->alpha;
      L.T_0 = p->T_0;
      L.TFACTOR = p->TFACTOR;
      L.moutlier = p->moutlier;
      L.form = form;
      L.dRt = dRt;
      L.trace = dtrace;
      L.trace_cap = cap;
      L.timeline = dtl;
      L.timeline_cap = tl_cap;
      L.timeout_ns = timeout_ns_of(p);
      kerr = enqueue_softassign(L, C.ws.p, C.ws.bytes, st, &grid);
    }
    cudaEventRecord(ev1, st);
    if (kerr != 0) e = (cudaError_t)kerr;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(hRt, dRt, sizeof(hRt), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int status = 0, steps = 0, tl_n = 0;
  if (e == cudaSuccess) e = (cudaError_t)read_ws_status(C.ws.p, st, &status, &steps, &tl_n);
  float ms = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (e != cudaSuccess) return map_cuda(e);
  if (status != 0) return status;
  C.last_kind = kind;
  C.last_trace_steps = steps < cap ? steps : cap;
  if (cap > 0 && C.last_trace_steps > 0) {
    e = cudaMemcpy(rep->trace, dtrace, sizeof(double) * 32 * (size_t)C.last_trace_steps,
                   cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return map_cuda(e);
  }
  if (tl_cap > 0) {
    // every block owns tl_cap / grid entries; unused entries stay zero
    e = cudaMemcpy(rep->timeline, dtl, sizeof(unsigned long long) * (size_t)tl_cap, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return map_cuda(e);
    rep->timeline_written = tl_n;
  }
  memcpy(R, hRt, sizeof(float) * 9);
  memcpy(t, hRt + 9, sizeof(float) * 3);
  if (rep) {
    rep->steps = (int)nsteps;
    rep->sinkhorn_form = form;
    rep->grid_blocks = grid;
    rep->device_ms = ms;
  }
  return CESA_OK;
}

// Validates a batch and converts it to launch records (device pointers are
// taken from the pairs unless dX/dY/dRt overrides are given).
int batch_records(const cesa_pair* pairs, int npairs, std::vector<BatchLaunchPair>& out) {
  if (!pairs || npairs < 1 || npairs > CESA_MAX_BATCH) return CESA_ERR_INVALID_ARGUMENT;
  out.resize((size_t)npairs);
  for (int i = 0; i < npairs; ++i) {
    const cesa_pair& q = pairs[i];
    int rc = check_points(q.X, q.N, q.Y, q.M);
    if (rc) return rc;
    if (!q.Rt) return CESA_ERR_INVALID_ARGUMENT;
    BatchLaunchPair& L = out[(size_t)i];
    L = BatchLaunchPair{};
    L.N = q.N;
    L.M = q.M;
    L.dX = q.X;
    L.dY = q.Y;
    L.dRt = q.Rt;
    if (q.algorithm == CESA_ALGO_EMICP) {
      rc = check_emicp_params(&q.params);
      if (rc) return rc;
      const long n = emicp_steps(q.params.sigma_p2, q.params.sigma_inf, q.params.sigma_factor);
      if (n < 0 || n > 1000000L) return CESA_ERR_INVALID_ARGUMENT;
      L.algo = 0;
      L.nsteps = (int)n;
      L.sigma_p2 = q.params.sigma_p2;
      L.sigma_factor = q.params.sigma_factor;
      L.d_02 = q.params.d_02;
    } else if (q.algorithm == CESA_ALGO_SOFTASSIGN) {
      rc = check_sa_params(&q.params);
      if (rc) return rc;
      if ((long)q.params.JMAX * q.params.I0 * (2L * q.params.I1 + 2) > 100000000L) return CESA_ERR_INVALID_ARGUMENT;
      L.algo = 1;
      L.JMAX = q.params.JMAX;
      L.I0 = q.params.I0;
      L.I1 = q.params.I1;
      L.alpha = q.params.alpha;
      L.T_0 = q.params.T_0;
      L.TFACTOR = q.params.TFACTOR;
      L.moutlier = q.params.moutlier;
    } else {
      return CESA_ERR_INVALID_ARGUMENT;
    }
  }
  return CESA_OK;
}

uint64_t batch_timeout_ns(const cesa_pair* pairs, int npairs) {
  uint64_t t = 0;
  for (int i = 0; i < npairs; ++i) {
    const uint64_t v = timeout_ns_of(&pairs[i].params);
    if (v > t) t = v;
  }
  return t;
}

}  // namespace

std::mutex& api_mutex() { return g_mu; }

void note_noalloc_call(int dev, cudaStream_t st, void* scratch) {
  NoallocRec* r = noalloc_rec(dev, st);
  if (!r) {
    r = &g_noalloc_rec[g_noalloc_next];
    g_noalloc_next = (g_noalloc_next + 1) % kNoallocRecs;
  }
  r->dev = dev;
  r->st = st;
  r->ctl = scratch;
}

}  // namespace cesa

using namespace cesa;

extern "C" {

void cesa_params_default(cesa_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->JMAX = 100;
  p->I0 = 5;
  p->I1 = 3;
  p->alpha = 3.0f;
  p->T_0 = 100.0f;
  p->TFACTOR = 0.95f;
  p->moutlier = (float)(1 / sqrtf(p->T_0) * expf(-1.0f));
  p->sigma_p2 = 0.01f;
  p->sigma_inf = 0.00001f;
  p->sigma_factor = 0.9f;
  p->d_02 = 0.01f;
  p->maxIteration = 30;
  p->sinkhorn_form = CESA_SINKHORN_AUTO;
  p->timeout_ms = 0;
  p->device = -1;
}

int cesa_emicp(const float* X, int N, const float* Y, int M, float R[9], float t[3],
               const cesa_params* p, cesa_report* rep) {
  return run_host(1, X, N, Y, M, R, t, p, rep);
}

int cesa_softassign(const float* X, int N, const float* Y, int M, float R[9], float t[3],
                    const cesa_params* p, cesa_report* rep) {
  return run_host(2, X, N, Y, M, R, t, p, rep);
}

int cesa_icp(const float* X, int N, const float* Y, int M, float R[9], float t[3], const cesa_params* p,
             cesa_report* rep) {
  return run_host(3, X, N, Y, M, R, t, p, rep);
}

int cesa_icp_device(const float* dX, int N, const float* dY, int M, float* dRt, const cesa_params* p,
                    int* d_nn, int* d_status, cesa_stream_t stream) {
  int rc = check_points(dX, N, dY, M);
  if (rc) return rc;
  if (!dRt) return CESA_ERR_INVALID_ARGUMENT;
  rc = check_icp_params(p);
  if (rc) return rc;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  cudaError_t e = C.ws.ensure(icp_ws_need(N, M, dev, p->icp_search));
  if (e != cudaSuccess) return map_cuda(e);
  IcpLaunch L{};
  L.dX = dX;
  L.dY = dY;
  L.N = N;
  L.M = M;
  L.iters = p->maxIteration;
  L.search = p->icp_search;
  L.dRt = dRt;
  L.nn_out = d_nn;
  L.d_status = d_status;
  L.timeout_ns = timeout_ns_of(p);
  C.last_kind = 3;
  C.last_trace_steps = 0;
  return map_cuda((cudaError_t)enqueue_icp(L, C.ws.p, C.ws.bytes, st, nullptr));
}

int cesa_emicp_device(const float* dX, int N, const float* dY, int M, float* dRt,
                      const cesa_params* p, int* d_status, cesa_stream_t stream) {
  int rc = check_points(dX, N, dY, M);
  if (rc) return rc;
  if (!dRt) return CESA_ERR_INVALID_ARGUMENT;
  rc = check_emicp_params(p);
  if (rc) return rc;
  const long nsteps = emicp_steps(p->sigma_p2, p->sigma_inf, p->sigma_factor);
  if (nsteps < 0) return CESA_ERR_INVALID_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  cudaError_t e = C.ws.ensure(emicp_ws_need(N, M, dev));
  if (e != cudaSuccess) return map_cuda(e);
  EmicpLaunch L{};
  L.dX = dX;
  L.dY = dY;
  L.N = N;
  L.M = M;
  L.sigma_p2 = p->sigma_p2;
  L.sigma_factor = p->sigma_factor;
  L.d_02 = p->d_02;
  L.nsteps = (int)nsteps;
  L.dRt = dRt;
  L.d_status = d_status;
  L.timeout_ns = timeout_ns_of(p);
  C.last_kind = 1;
  C.last_trace_steps = 0;
  return map_cuda((cudaError_t)enqueue_emicp(L, C.ws.p, C.ws.bytes, st, nullptr));
}

int cesa_softassign_device(const float* dX, int N, const float* dY, int M, float* dRt,
                           const cesa_params* p, int* d_status, cesa_stream_t stream) {
  int rc = check_points(dX, N, dY, M);
  if (rc) return rc;
  if (!dRt) return CESA_ERR_INVALID_ARGUMENT;
  rc = check_sa_params(p);
  if (rc) return rc;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  const int form = resolve_form(p->sinkhorn_form, N, M, dev);
  cudaError_t e = C.ws.ensure(softassign_ws_need(N, M, form, dev));
  if (e != cudaSuccess) return map_cuda(e);
  SoftassignLaunch L{};
  L.dX = dX;
  L.dY = dY;
  L.N = N;
  L.M = M;
  L.JMAX = p->JMAX;
  L.I0 = p->I0;
  L.I1 = p->I1;
  L.alpha = p->alpha;
  L.T_0 = p->T_0;
  L.TFACTOR = p->TFACTOR;
  L.moutlier = p->moutlier;
  L.form = form;
  L.dRt = dRt;
  L.d_status = d_status;
  L.timeout_ns = timeout_ns_of(p);
  C.last_kind = 2;
  C.last_trace_steps = 0;
  return map_cuda((cudaError_t)enqueue_softassign(L, C.ws.p, C.ws.bytes, st, nullptr));
}

int cesa_register_batch_device(const cesa_pair* pairs, int npairs, int* d_status, cesa_stream_t stream) {
  std::vector<BatchLaunchPair> rec;
  int rc = batch_records(pairs, npairs, rec);
  if (rc) return rc;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  cudaError_t e = C.ws.ensure(batch_ws_need(rec.data(), npairs, dev));
  if (e != cudaSuccess) return map_cuda(e);
  C.last_kind = 3;
  C.last_trace_steps = 0;
  return map_cuda((cudaError_t)enqueue_batch(rec.data(), npairs, d_status, batch_timeout_ns(pairs, npairs),
                                             C.ws.p, C.ws.bytes, st, nullptr, nullptr));
}

int cesa_register_batch(const cesa_pair* pairs, int npairs, cesa_report* rep) {
  std::vector<BatchLaunchPair> rec;
  int rc = batch_records(pairs, npairs, rec);
  if (rc) return rc;
  int dev = 0;
  rc = select_device(&pairs[0].params, &dev);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t st = own_stream(dev);
  StreamCtx& C = ctx_for(dev, st);
  // device copies: X, Y of every pair, then the poses
  std::vector<size_t> ox((size_t)npairs), oy((size_t)npairs);
  size_t off = 0;
  for (int i = 0; i < npairs; ++i) {
    ox[(size_t)i] = off;
    off += align256(sizeof(float) * 3 * (size_t)pairs[i].N);
    oy[(size_t)i] = off;
    off += align256(sizeof(float) * 3 * (size_t)pairs[i].M);
  }
  const size_t opose = off;
  off += align256(sizeof(float) * 12 * (size_t)npairs);
  cudaError_t e = C.io.ensure(off);
  if (e != cudaSuccess) return map_cuda(e);
  char* io = static_cast<char*>(C.io.p);
  float* dpose = reinterpret_cast<float*>(io + opose);
  std::vector<float> hpose((size_t)npairs * 12);
  for (int i = 0; i < npairs; ++i) {
    BatchLaunchPair& L = rec[(size_t)i];
    float* dx = reinterpret_cast<float*>(io + ox[(size_t)i]);
    float* dy = reinterpret_cast<float*>(io + oy[(size_t)i]);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dx, pairs[i].X, sizeof(float) * 3 * (size_t)L.N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dy, pairs[i].Y, sizeof(float) * 3 * (size_t)L.M, cudaMemcpyHostToDevice, st);
    L.dX = dx;
    L.dY = dy;
    L.dRt = dpose + (size_t)i * 12;
    memcpy(&hpose[(size_t)i * 12], pairs[i].Rt, sizeof(float) * 12);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dpose, hpose.data(), sizeof(float) * hpose.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = C.ws.ensure(batch_ws_need(rec.data(), npairs, dev));
  if (e != cudaSuccess) return map_cuda(e);
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  int grid = 0, rounds = 0;
  cudaEventRecord(ev0, st);
  int kerr = enqueue_batch(rec.data(), npairs, nullptr, batch_timeout_ns(pairs, npairs), C.ws.p, C.ws.bytes, st,
                           &grid, &rounds);
  cudaEventRecord(ev1, st);
  if (kerr != 0) e = (cudaError_t)kerr;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(hpose.data(), dpose, sizeof(float) * hpose.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  int status = 0, steps = 0;
  if (e == cudaSuccess) e = (cudaError_t)read_ws_status(C.ws.p, st, &status, &steps);
  float ms = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (e != cudaSuccess) return map_cuda(e);
  if (status != 0) return status;
  C.last_kind = 3;
  C.last_trace_steps = 0;
  for (int i = 0; i < npairs; ++i) memcpy(pairs[i].Rt, &hpose[(size_t)i * 12], sizeof(float) * 12);
  if (rep) {
    rep->steps = rounds;
    rep->sinkhorn_form = CESA_SINKHORN_MATRIX_FREE;
    rep->grid_blocks = grid;
    rep->device_ms = ms;
  }
  return CESA_OK;
}

}  // extern "C"

namespace {
// Layout of an EM-ICP tape buffer: centring header, packed X' and Y', the
// step records, the per-step row records.
struct TapeLayout {
  size_t hdr, cols, rows, steps, row_tape, total;
};
TapeLayout tape_layout(int N, int M, long nsteps) {
  TapeLayout t;
  size_t off = 0;
  t.hdr = off;
  off += align256(sizeof(CenterHdr));
  t.cols = off;
  off += align256(sizeof(float4) * (size_t)N);
  t.rows = off;
  off += align256(sizeof(float4) * (size_t)M);
  t.steps = off;
  off += align256(sizeof(float) * kEmTape * (size_t)nsteps);
  t.row_tape = off;
  off += align256(sizeof(float) * 5 * (size_t)M * (size_t)nsteps);
  t.total = off;
  return t;
}
// Softassign tape: header, packed clouds, and per pose update its record
// (kSaTape floats: input pose, sumM, centres, S, Horn's solve), the input slack
// s (N) and u (M), the row- and column-pass vectors ([I1][4][N], [I1][4][M])
// and the final sweep's row sums ([5][N]).
struct SaTapeLayout {
  size_t hdr, X, Y, pose, s, u, rows, cols, fin, total;
};
SaTapeLayout sa_tape_layout(int N, int M, int I1, long nsteps) {
  SaTapeLayout t;
  size_t off = 0;
  auto put = [&off](size_t bytes) {
    const size_t at = off;
    off += align256(bytes);
    return at;
  };
  const size_t n = (size_t)nsteps;
  t.hdr = put(sizeof(CenterHdr));
  t.X = put(sizeof(float4) * (size_t)N);
  t.Y = put(sizeof(float4) * (size_t)M);
  t.pose = put(sizeof(float) * kSaTape * n);
  t.s = put(sizeof(float) * (size_t)N * n);
  t.u = put(sizeof(float) * (size_t)M * n);
  t.rows = put(sizeof(float) * (size_t)I1 * 4 * N * n);
  t.cols = put(sizeof(float) * (size_t)I1 * 4 * M * n);
  t.fin = put(sizeof(float) * 5 * (size_t)N * n);
  t.total = off;
  return t;
}
}  // namespace

extern "C" {

size_t cesa_emicp_tape_bytes(int N, int M, const cesa_params* p) {
  if (N < 1 || M < 1 || check_emicp_params(p)) return 0;
  const long n = emicp_steps(p->sigma_p2, p->sigma_inf, p->sigma_factor);
  if (n < 0) return 0;
  return tape_layout(N, M, n).total;
}

int cesa_emicp_forward_device(const float* dX, int N, const float* dY, int M, float* dRt, const cesa_params* p,
                              void* tape, int* d_status, cesa_stream_t stream) {
  int rc = check_points(dX, N, dY, M);
  if (rc) return rc;
  if (!dRt || !tape) return CESA_ERR_INVALID_ARGUMENT;
  rc = check_emicp_params(p);
  if (rc) return rc;
  const long nsteps = emicp_steps(p->sigma_p2, p->sigma_inf, p->sigma_factor);
  if (nsteps < 0) return CESA_ERR_INVALID_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  cudaError_t e = C.ws.ensure(emicp_ws_need(N, M, dev));
  if (e != cudaSuccess) return map_cuda(e);
  const TapeLayout T = tape_layout(N, M, nsteps);
  char* tb = static_cast<char*>(tape);
  EmicpLaunch L{};
  L.dX = dX;
  L.dY = dY;
  L.N = N;
  L.M = M;
  L.sigma_p2 = p->sigma_p2;
  L.sigma_factor = p->sigma_factor;
  L.d_02 = p->d_02;
  L.nsteps = (int)nsteps;
  L.dRt = dRt;
  L.d_status = d_status;
  L.timeout_ns = timeout_ns_of(p);
  L.tape = reinterpret_cast<float*>(tb + T.steps);
  L.row_tape = reinterpret_cast<float*>(tb + T.row_tape);
  C.last_kind = 1;
  C.last_trace_steps = 0;
  int k = enqueue_emicp(L, C.ws.p, C.ws.bytes, st, nullptr);
  if (k) return map_cuda((cudaError_t)k);
  // the packed clouds and offsets the forward used
  CenterHdr* hdr = nullptr;
  float4 *rows = nullptr, *cols = nullptr;
  emicp_ws_views(C.ws.p, N, M, dev, &hdr, &rows, &cols);
  e = cudaMemcpyAsync(tb + T.hdr, hdr, sizeof(CenterHdr), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tb + T.cols, cols, sizeof(float4) * (size_t)N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tb + T.rows, rows, sizeof(float4) * (size_t)M, cudaMemcpyDeviceToDevice, st);
  return map_cuda(e);
}

int cesa_emicp_backward_device(int N, int M, const cesa_params* p, const void* tape, const float* d_gRt,
                               float* d_gX, float* d_gY, float* d_gRt0, int* d_status, cesa_stream_t stream) {
  if (N < 1 || M < 1 || !tape || !d_gRt || !d_gX || !d_gY || !d_gRt0) return CESA_ERR_INVALID_ARGUMENT;
  int rc = check_emicp_params(p);
  if (rc) return rc;
  if (p->emicp_backward_layout < CESA_LAYOUT_AUTO || p->emicp_backward_layout > CESA_LAYOUT_RANGED)
    return CESA_ERR_INVALID_ARGUMENT;
  const long nsteps = emicp_steps(p->sigma_p2, p->sigma_inf, p->sigma_factor);
  if (nsteps < 0) return CESA_ERR_INVALID_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  cudaError_t e = C.ws.ensure(emicp_adjoint_ws_need(N, M, dev, p->emicp_backward_layout));
  if (e != cudaSuccess) return map_cuda(e);
  const TapeLayout T = tape_layout(N, M, nsteps);
  const char* tb = static_cast<const char*>(tape);
  EmicpAdjointLaunch L{};
  L.rows = reinterpret_cast<const float4*>(tb + T.rows);
  L.cols = reinterpret_cast<const float4*>(tb + T.cols);
  L.hdr = reinterpret_cast<const CenterHdr*>(tb + T.hdr);
  L.N = N;
  L.M = M;
  L.nsteps = (int)nsteps;
  L.tape = reinterpret_cast<const float*>(tb + T.steps);
  L.row_tape = reinterpret_cast<const float*>(tb + T.row_tape);
  L.g_out = d_gRt;
  L.gX = d_gX;
  L.gY = d_gY;
  L.g_in = d_gRt0;
  L.d_status = d_status;
  L.timeout_ns = timeout_ns_of(p);
  L.layout = p->emicp_backward_layout;
  C.last_kind = 1;
  C.last_trace_steps = 0;
  return map_cuda((cudaError_t)enqueue_emicp_adjoint(L, C.ws.p, C.ws.bytes, st));
}

size_t cesa_softassign_tape_bytes(int N, int M, const cesa_params* p) {
  if (N < 1 || M < 1 || check_sa_params(p)) return 0;
  return sa_tape_layout(N, M, p->I1, (long)p->JMAX * p->I0).total;
}

int cesa_softassign_forward_device(const float* dX, int N, const float* dY, int M, float* dRt, const cesa_params* p,
                                   void* tape, int* d_status, cesa_stream_t stream) {
  int rc = check_points(dX, N, dY, M);
  if (rc) return rc;
  if (!dRt || !tape) return CESA_ERR_INVALID_ARGUMENT;
  rc = check_sa_params(p);
  if (rc) return rc;
  const long nsteps = (long)p->JMAX * p->I0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  cudaError_t e = C.ws.ensure(softassign_ws_need(N, M, kFormMatrixFree, dev));
  if (e != cudaSuccess) return map_cuda(e);
  const SaTapeLayout T = sa_tape_layout(N, M, p->I1, nsteps);
  char* tb = static_cast<char*>(tape);
  SoftassignLaunch L{};
  L.dX = dX;
  L.dY = dY;
  L.N = N;
  L.M = M;
  L.JMAX = p->JMAX;
  L.I0 = p->I0;
  L.I1 = p->I1;
  L.alpha = p->alpha;
  L.T_0 = p->T_0;
  L.TFACTOR = p->TFACTOR;
  L.moutlier = p->moutlier;
  L.form = kFormMatrixFree;  // the tape is recorded by the matrix-free kernel
  L.dRt = dRt;
  L.d_status = d_status;
  L.timeout_ns = timeout_ns_of(p);
  L.tape_pose = reinterpret_cast<float*>(tb + T.pose);
  L.tape_s = reinterpret_cast<float*>(tb + T.s);
  L.tape_u = reinterpret_cast<float*>(tb + T.u);
  L.tape_rows = reinterpret_cast<float*>(tb + T.rows);
  L.tape_cols = reinterpret_cast<float*>(tb + T.cols);
  L.tape_fin = reinterpret_cast<float*>(tb + T.fin);
  C.last_kind = 2;
  C.last_trace_steps = 0;
  const int k = enqueue_softassign(L, C.ws.p, C.ws.bytes, st, nullptr);
  if (k) return map_cuda((cudaError_t)k);
  CenterHdr* hdr = nullptr;
  float4 *rows = nullptr, *cols = nullptr;
  softassign_ws_views(C.ws.p, N, M, dev, &hdr, &rows, &cols);
  e = cudaMemcpyAsync(tb + T.hdr, hdr, sizeof(CenterHdr), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tb + T.X, rows, sizeof(float4) * (size_t)N, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tb + T.Y, cols, sizeof(float4) * (size_t)M, cudaMemcpyDeviceToDevice, st);
  return map_cuda(e);
}

int cesa_softassign_backward_device(int N, int M, const cesa_params* p, const void* tape, const float* d_gRt,
                                    float* d_gX, float* d_gY, float* d_gRt0, int* d_status, cesa_stream_t stream) {
  if (N < 1 || M < 1 || !tape || !d_gRt || !d_gX || !d_gY || !d_gRt0) return CESA_ERR_INVALID_ARGUMENT;
  int rc = check_sa_params(p);
  if (rc) return rc;
  if (p->softassign_backward_form < CESA_SA_BACKWARD_AUTO || p->softassign_backward_form > CESA_SA_BACKWARD_LAUNCHES)
    return CESA_ERR_INVALID_ARGUMENT;
  const long nsteps = (long)p->JMAX * p->I0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  const size_t need = softassign_bwd_ws_need(N, M, p->I1, nsteps);
  if (C.ws.bytes < need) C.sa_bwd.release();  // its graph refers to the old workspace
  cudaError_t e = C.ws.ensure(need);
  if (e != cudaSuccess) return map_cuda(e);
  const SaTapeLayout T = sa_tape_layout(N, M, p->I1, nsteps);
  const char* tb = static_cast<const char*>(tape);
  SoftassignBackward B{};
  B.X = reinterpret_cast<const float4*>(tb + T.X);
  B.Y = reinterpret_cast<const float4*>(tb + T.Y);
  B.hdr = reinterpret_cast<const CenterHdr*>(tb + T.hdr);
  B.N = N;
  B.M = M;
  B.I1 = p->I1;
  B.nsteps = nsteps;
  B.alpha = p->alpha;
  B.g_out = d_gRt;
  B.gX = d_gX;
  B.gY = d_gY;
  B.g_in = d_gRt0;
  // the updates' tape slices and temperatures (T stepped in FP32 as the forward does)
  std::vector<SaUpdate> tab((size_t)nsteps);
  {
    const size_t I1 = (size_t)p->I1;
    float Tk = p->T_0;
    size_t k = 0;
    for (int j = 0; j < p->JMAX; ++j) {
      for (int i = 0; i < p->I0; ++i, ++k) {
        SaUpdate& U = tab[k];
        U.rec = reinterpret_cast<const float*>(tb + T.pose) + k * kSaTape;
        U.s0 = reinterpret_cast<const float*>(tb + T.s) + k * N;
        U.u0 = reinterpret_cast<const float*>(tb + T.u) + k * M;
        U.rows = reinterpret_cast<const float*>(tb + T.rows) + k * I1 * 4 * N;
        U.cols = reinterpret_cast<const float*>(tb + T.cols) + k * I1 * 4 * M;
        U.fin = reinterpret_cast<const float*>(tb + T.fin) + k * 5 * N;
        U.T = Tk;
      }
      Tk = Tk * p->TFACTOR;
    }
  }
  C.last_kind = 2;
  C.last_trace_steps = 0;
  // Small problems, whose updates are latency-bound chains of small stages:
  // one persistent launch over all updates (measured at N = M = 2000: 101 us
  // per update, against 142 us replayed as a graph). Large ones are
  // work-bound and run the per-update launch sequence, whose sweeps hold more
  // warps per SM (N = M = 20,000: 1.46 ms per update, against 1.57 ms in the
  // persistent kernel). The sequence also stands in where the persistent
  // kernel cannot launch.
  int r = (int)cudaErrorCooperativeLaunchTooLarge;
  const int form = p->softassign_backward_form;
  const bool persistent = form == CESA_SA_BACKWARD_PERSISTENT ||
                          (form == CESA_SA_BACKWARD_AUTO && (double)N * (double)M <= kSaBwdPersistentMaxElems);
  if (persistent) r = softassign_bwd_persistent(B, tab.data(), C.ws.p, C.ws.bytes, st, d_status, timeout_ns_of(p));
  if (r != (int)cudaErrorCooperativeLaunchTooLarge) return map_cuda((cudaError_t)r);
  cudaGetLastError();
  r = softassign_bwd_prepare(B, tab.data(), C.ws.p, C.ws.bytes, st);
  if (r) return map_cuda((cudaError_t)r);
  // one update's launches as a graph (captured once per workspace layout), replayed per update
  SaBwdGraph& G = C.sa_bwd;
  bool graphed = false;
  if (nsteps > 0) {
    const bool same = G.exec && G.ws == C.ws.p && G.bytes == C.ws.bytes && G.N == N && G.M == M && G.I1 == p->I1 &&
                      G.alpha == p->alpha;
    if (!same) {
      G.release();
      if (cudaStreamCreateWithFlags(&G.stream, cudaStreamNonBlocking) == cudaSuccess &&
          cudaEventCreateWithFlags(&G.fork, cudaEventDisableTiming) == cudaSuccess &&
          cudaEventCreateWithFlags(&G.join, cudaEventDisableTiming) == cudaSuccess &&
          cudaStreamBeginCapture(G.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int ur = softassign_bwd_update(B, C.ws.p, C.ws.bytes, G.stream);
        cudaGraph_t graph = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(G.stream, &graph);
        if (ur == 0 && ce == cudaSuccess && graph &&
            cudaGraphInstantiate(&G.exec, graph, 0) == cudaSuccess) {
          G.ws = C.ws.p;
          G.bytes = C.ws.bytes;
          G.N = N;
          G.M = M;
          G.I1 = p->I1;
          G.alpha = p->alpha;
        } else {
          G.exec = nullptr;
        }
        if (graph) cudaGraphDestroy(graph);
      }
      cudaGetLastError();  // a failed capture leaves the direct launches below
      if (!G.exec) G.release();
    }
    if (G.exec) {
      e = cudaEventRecord(G.fork, st);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(G.stream, G.fork, 0);
      for (long n = 0; n < nsteps && e == cudaSuccess; ++n) e = cudaGraphLaunch(G.exec, G.stream);
      if (e == cudaSuccess) e = cudaEventRecord(G.join, G.stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, G.join, 0);
      if (e != cudaSuccess) return map_cuda(e);
      graphed = true;
    }
  }
  if (!graphed)
    for (long n = 0; n < nsteps; ++n) {
      r = softassign_bwd_update(B, C.ws.p, C.ws.bytes, st);
      if (r) return map_cuda((cudaError_t)r);
    }
  r = softassign_bwd_finish(B, C.ws.p, C.ws.bytes, st);
  if (r) return map_cuda((cudaError_t)r);
  // the launch sequence has no device-side waits: its status is set once all launches are queued
  if (d_status) e = cudaMemsetAsync(d_status, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(C.ws.p, 0, sizeof(int) * 4, st);  // the control block: CESA_OK
  return map_cuda(e);
}

int cesa_tune_sinkhorn(int N, int M, const cesa_params* p, int* form_out, float* ms_matrix_free,
                       float* ms_materialised) {
  if (N < 1 || M < 1 || (long)N * 16 > 0x7fffffffL || (long)M * 16 > 0x7fffffffL) return CESA_ERR_INVALID_ARGUMENT;
  cesa_params q;
  if (p) {
    q = *p;
  } else {
    cesa_params_default(&q);
  }
  if (check_sa_params(&q)) return CESA_ERR_INVALID_ARGUMENT;
  int dev = 0;
  int rc = select_device(&q, &dev);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(g_mu);
  cudaStream_t st = own_stream(dev);
  // synthetic clouds of the requested sizes (timing does not depend on the
  // values: the sweeps have no data-dependent branches)
  std::vector<float> hx(3 * (size_t)N), hy(3 * (size_t)M);
  unsigned long long z = 0x9e3779b97f4a7c15ull;
  auto next = [&z]() {
    z = z * 6364136223846793005ull + 1442695040888963407ull;
    return (float)((z >> 40) & 0xffffff) / 16777216.f;
  };
  for (auto& v : hx) v = next();
  for (auto& v : hy) v = next();
  const bool try_mat = materialised_fits(N, M);
  const bool try_band = softassign_band_fits(N, M, dev);
  const size_t need_f = softassign_ws_need(N, M, kFormMatrixFree, dev);
  const size_t need_m = try_mat ? softassign_ws_need(N, M, kFormMaterialised, dev) : 0;
  const size_t need_b = try_band ? softassign_ws_need(N, M, kFormBanded, dev) : 0;
  size_t need = need_f > need_m ? need_f : need_m;
  if (need_b > need) need = need_b;
  void* mem = nullptr;
  const size_t bx = align256(sizeof(float) * hx.size()), by = align256(sizeof(float) * hy.size());
  cudaError_t e = cudaMalloc(&mem, bx + by + 256 + need);
  if (e != cudaSuccess) return map_cuda(e);
  char* base = static_cast<char*>(mem);
  float* dX = reinterpret_cast<float*>(base);
  float* dY = reinterpret_cast<float*>(base + bx);
  float* dRt = reinterpret_cast<float*>(base + bx + by);
  void* ws = base + bx + by + 256;
  const float pose[12] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0};
  e = cudaMemcpyAsync(dX, hx.data(), sizeof(float) * hx.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dY, hy.data(), sizeof(float) * hy.size(), cudaMemcpyHostToDevice, st);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms[3] = {-1.f, -1.f, -1.f};  // matrix-free, materialised, banded
  for (int f = 0; f < 3 && e == cudaSuccess; ++f) {
    const int form = f == 0 ? kFormMatrixFree : f == 1 ? kFormMaterialised : kFormBanded;
    if ((form == kFormMaterialised && !try_mat) || (form == kFormBanded && !try_band)) continue;
    SoftassignLaunch L{};
    L.dX = dX;
    L.dY = dY;
    L.N = N;
    L.M = M;
    L.JMAX = 1;
    L.I0 = 2;
    L.I1 = q.I1;
    L.alpha = q.alpha;
    L.T_0 = q.T_0;
    L.TFACTOR = q.TFACTOR;
    L.moutlier = q.moutlier;
    L.form = form;
    L.dRt = dRt;
    L.timeout_ns = timeout_ns_of(&q);
    float best = 0.f;
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {  // first run is the warm-up
      e = cudaMemcpyAsync(dRt, pose, sizeof(pose), cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaEventRecord(e0, st);
      if (e == cudaSuccess) e = (cudaError_t)enqueue_softassign(L, ws, need, st, nullptr);
      if (e == cudaSuccess) e = cudaEventRecord(e1, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float t = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
      if (rep == 1 || (rep > 1 && t < best)) best = t;
    }
    int status = 0, steps = 0;
    if (e == cudaSuccess) e = (cudaError_t)read_ws_status(ws, st, &status, &steps);
    if (e == cudaSuccess && status) rc = status;
    ms[f] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamSynchronize(st);
  cudaFree(mem);
  if (e != cudaSuccess) return map_cuda(e);
  if (rc) return rc;
  // matrix-free arithmetic: the faster of its two decompositions; the
  // materialised form also holds N x M floats: it must win by 10%
  const bool band_wins = ms[2] >= 0.f && ms[2] < ms[0];
  const float ms_free = band_wins ? ms[2] : ms[0];
  const int form = (ms[1] >= 0.f && ms[1] < 0.9f * ms_free) ? kFormMaterialised
                   : band_wins                               ? kFormBanded
                                                             : kFormMatrixFree;
  g_tuned[TuneKey{dev, size_bucket(N), size_bucket(M)}] = form;
  if (form_out) *form_out = form;
  if (ms_matrix_free) *ms_matrix_free = ms_free * 0.5f;  // per pose update
  if (ms_materialised) *ms_materialised = ms[1] >= 0.f ? ms[1] * 0.5f : -1.f;
  return CESA_OK;
}

int cesa_stream_status(cesa_stream_t stream) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lock(g_mu);
  void* ctl = nullptr;
  if (NoallocRec* r = noalloc_rec(dev, (cudaStream_t)stream)) {
    ctl = r->ctl;
  } else {
    auto it = g_ctx.find(std::make_pair(dev, (cudaStream_t)stream));
    if (it != g_ctx.end()) ctl = it->second.ws.p;
  }
  if (!ctl) return CESA_ERR_INVALID_ARGUMENT;
  int status = 0, steps = 0;
  const int e = read_ws_status(ctl, (cudaStream_t)stream, &status, &steps);
  if (e) return map_cuda((cudaError_t)e);
  return status;
}

int cesa_emicp_step_device(const float* dX, int N, const float* dY, int M, const float R[9],
                           const float t[3], float sigma_p2, float d_02, float* row_out,
                           double moments[16], cesa_stream_t stream) {
  int rc = check_points(dX, N, dY, M);
  if (rc) return rc;
  if (!R || !t || !(sigma_p2 > 0.f) || !(d_02 >= 0.f)) return CESA_ERR_INVALID_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  cudaError_t e = C.ws.ensure(emicp_ws_need(N, M, dev));
  if (e == cudaSuccess) e = C.io.ensure(256);
  if (e == cudaSuccess) e = C.trace.ensure(sizeof(double) * 32);
  if (e != cudaSuccess) return map_cuda(e);
  float hRt[12];
  memcpy(hRt, R, sizeof(float) * 9);
  memcpy(hRt + 9, t, sizeof(float) * 3);
  float* dRt = static_cast<float*>(C.io.p);
  e = cudaMemcpyAsync(dRt, hRt, sizeof(hRt), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return map_cuda(e);
  EmicpLaunch L{};
  L.dX = dX;
  L.dY = dY;
  L.N = N;
  L.M = M;
  L.sigma_p2 = sigma_p2;
  L.sigma_factor = 1.f;
  L.d_02 = d_02;
  L.nsteps = 1;
  L.dRt = dRt;
  L.row_out = row_out;
  L.trace = static_cast<double*>(C.trace.p);
  L.trace_cap = 1;
  L.timeout_ns = 10000000000ull;
  const int k = enqueue_emicp(L, C.ws.p, C.ws.bytes, st, nullptr);
  if (k) return map_cuda((cudaError_t)k);
  double rec[32];
  e = cudaMemcpyAsync(rec, C.trace.p, sizeof(rec), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return map_cuda(e);
  int status = 0, steps = 0;
  read_ws_status(C.ws.p, st, &status, &steps);
  if (status) return status;
  if (moments) {
    moments[0] = rec[2];
    for (int i = 0; i < 3; ++i) {
      moments[1 + i] = rec[3 + i];
      moments[4 + i] = rec[6 + i];
    }
    for (int i = 0; i < 9; ++i) moments[7 + i] = rec[9 + i];
  }
  return CESA_OK;
}

int cesa_softassign_step_device(const float* dX, int N, const float* dY, int M, const float R[9],
                                const float t[3], float T, float alpha, int I1, int sinkhorn_form,
                                float* s, float* u, float* rs, float* cs, float* w,
                                double moments[16], cesa_stream_t stream) {
  int rc = check_points(dX, N, dY, M);
  if (rc) return rc;
  if (!R || !t || !s || !u || !(T > 0.f) || I1 < 1) return CESA_ERR_INVALID_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mu);
  StreamCtx& C = ctx_for(dev, st);
  const int form = resolve_form(sinkhorn_form, N, M, dev);
  cudaError_t e = C.ws.ensure(softassign_ws_need(N, M, form, dev));
  if (e == cudaSuccess) e = C.io.ensure(256);
  if (e == cudaSuccess) e = C.trace.ensure(sizeof(double) * 32);
  if (e != cudaSuccess) return map_cuda(e);
  float hRt[12];
  memcpy(hRt, R, sizeof(float) * 9);
  memcpy(hRt + 9, t, sizeof(float) * 3);
  float* dRt = static_cast<float*>(C.io.p);
  e = cudaMemcpyAsync(dRt, hRt, sizeof(hRt), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return map_cuda(e);
  SoftassignLaunch L{};
  L.dX = dX;
  L.dY = dY;
  L.N = N;
  L.M = M;
  L.JMAX = 1;
  L.I0 = 1;
  L.I1 = I1;
  L.alpha = alpha;
  L.T_0 = T;
  L.TFACTOR = 1.f;
  L.moutlier = 0.f;
  L.form = form;
  L.dRt = dRt;
  L.s_io = s;
  L.u_io = u;
  L.rs_out = rs;
  L.cs_out = cs;
  L.w_out = w;
  L.trace = static_cast<double*>(C.trace.p);
  L.trace_cap = 1;
  L.timeout_ns = 10000000000ull;
  const int k = enqueue_softassign(L, C.ws.p, C.ws.bytes, st, nullptr);
  if (k) return map_cuda((cudaError_t)k);
  double rec[32];
  e = cudaMemcpyAsync(rec, C.trace.p, sizeof(rec), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return map_cuda(e);
  int status = 0, steps = 0;
  read_ws_status(C.ws.p, st, &status, &steps);
  if (status) return status;
  if (moments) {
    moments[0] = rec[2];
    for (int i = 0; i < 3; ++i) {
      moments[1 + i] = rec[3 + i];
      moments[4 + i] = rec[6 + i];
    }
    for (int i = 0; i < 9; ++i) moments[7 + i] = rec[9 + i];
  }
  return CESA_OK;
}

int cesa_find_rt_from_s(const float Xc[3], const float Yc[3], const float S[9], float R[9],
                        float t[3], float q_prev[4]) {
  if (!Xc || !Yc || !S || !R || !t) return CESA_ERR_INVALID_ARGUMENT;
  HornState<double> st;
  st.reset();
  if (q_prev)
    for (int i = 0; i < 4; ++i) st.q[i] = q_prev[i];
  double Sd[9], q[4], gap, lmax;
  for (int i = 0; i < 9; ++i) Sd[i] = S[i];
  const int fb = horn_quaternion<double>(Sd, st, q, &gap, &lmax);
  // R from the FP32-rounded quaternion, t = Xc - R Yc in FP32, as the
  // reference does with its float q (src/findRTfromS.cpp:57,80-96).
  float qf[4];
  for (int i = 0; i < 4; ++i) qf[i] = (float)q[i];
  float xc[3] = {Xc[0], Xc[1], Xc[2]}, yc[3] = {Yc[0], Yc[1], Yc[2]};
  quat_to_pose<float>(qf, xc, yc, R, t);
  if (q_prev && !fb)
    for (int i = 0; i < 4; ++i) q_prev[i] = qf[i];
  return CESA_OK;
}

int cesa_cloud2data(const float* points, int n, int stride_floats, float* soa_out) {
  if (n < 0 || (n > 0 && (!points || !soa_out)) || stride_floats < 3) return CESA_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < n; ++i) {
    soa_out[i] = points[(size_t)i * stride_floats + 0];
    soa_out[n + i] = points[(size_t)i * stride_floats + 1];
    soa_out[2 * n + i] = points[(size_t)i * stride_floats + 2];
  }
  return CESA_OK;
}

void cesa_release_workspaces(void) {
  std::lock_guard<std::mutex> lock(g_mu);
  for (auto& kv : g_ctx) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(kv.first.first);
    kv.second.sa_bwd.release();
    kv.second.ws.release();
    kv.second.io.release();
    kv.second.trace.release();
    kv.second.tl.release();
    cudaSetDevice(cur);
  }
  g_ctx.clear();
}

const char* cesa_status_string(int status) {
  switch (status) {
    case CESA_OK: return "ok";
    case CESA_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CESA_ERR_CUDA: return "CUDA runtime error";
    case CESA_ERR_TIMEOUT: return "device-side wait timed out";
    case CESA_ERR_NO_DEVICE: return "no usable CUDA device";
    case CESA_ERR_OUT_OF_MEMORY: return "out of memory";
    case CESA_ERR_UNSUPPORTED: return "unsupported request";
    case CESA_ERR_NOALLOC_LIMIT: return "problem exceeds the 16 MiB fixed scratch of cesa_emicp_device_noalloc";
    case CESA_ERR_INTERNAL: return "internal consistency check failed in a kernel (the access was skipped)";
    default: return "unknown status";
  }
}

int cesa_version(void) { return 100; }

}  // extern "C"
