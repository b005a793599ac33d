// cesa_emicp_device_noalloc: EM-ICP for callers that cannot allocate device
// memory.
//
// Some callers must not call cudaMalloc. A plugin inside a host application may
// own no device heap. A pre-sized real-time pipeline may forbid allocation after
// start-up.
// cesa_emicp_device() takes its workspace from a cudaMalloc'd cache. This entry
// point runs the same fused EM-ICP kernels on a fixed scratch array instead: a
// file-scope __device__ array of kNoAllocScratchBytes that every GPU which loads
// this library holds until the process exits.
//
// The caller still passes the inputs (device SoA X, Y) and the in/out pose.
// Nothing here calls cudaMalloc, cudaFree or an allocating library routine.
#include <cuda_runtime.h>
#include <mutex>

#include "../../include/cesa.h"
#include "cesa_kernels.h"

namespace {

// 16 MiB covers the EM-ICP workspace up to about N = M = 100,000 points.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};  // guarded by cesa::api_mutex()

}  // namespace

extern "C" int cesa_emicp_device_noalloc(const float* dX, int N, const float* dY, int M, float* dRt,
                                         const cesa_params* p, int* d_status, cesa_stream_t stream) {
  int rc = cesa::check_points(dX, N, dY, M);
  if (rc) return rc;
  if (!dRt) return CESA_ERR_INVALID_ARGUMENT;
  rc = cesa::check_emicp_params(p);
  if (rc) return rc;
  const long nsteps = cesa::emicp_steps(p->sigma_p2, p->sigma_inf, p->sigma_factor);
  if (nsteps < 0) return CESA_ERR_INVALID_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CESA_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return CESA_ERR_UNSUPPORTED;
  cudaStream_t st = (cudaStream_t)stream;
  // The same lock as every other entry point: the plan behind the size check
  // and the launch is made once, for this device.
  std::lock_guard<std::mutex> lock(cesa::api_mutex());
  if (cesa::emicp_ws_need(N, M, dev) > kNoAllocScratchBytes) return CESA_ERR_NOALLOC_LIMIT;
  if (!g_scratch_addr[dev]) {
    // The name g_noalloc_scratch is a host-side stand-in here, not a device
    // address. Resolve the device address once per device, with that device
    // current.
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return CESA_ERR_CUDA;
    g_scratch_addr[dev] = ptr;
  }
  void* scratch = g_scratch_addr[dev];
  cesa::EmicpLaunch L{};
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
  L.timeout_ns = cesa::timeout_ns_of(p);
  // enqueue_emicp clears the control block and split counters in the scratch
  // (cudaMemsetAsync, no allocation) before its kernels run.
  const int e = cesa::enqueue_emicp(L, scratch, kNoAllocScratchBytes, st, nullptr);
  if (e != (int)cudaSuccess)
    return e == (int)cudaErrorCooperativeLaunchTooLarge ? CESA_ERR_UNSUPPORTED : CESA_ERR_CUDA;
  // cesa_stream_status(stream) now reads this call's status from the scratch.
  cesa::note_noalloc_call(dev, st, scratch);
  return CESA_OK;
}
