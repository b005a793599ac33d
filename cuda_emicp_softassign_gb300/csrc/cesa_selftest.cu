// cesa_self_test_waits: runs the bounded waits of the registration kernels on
// barriers that nothing completes and reports the status they leave behind.
// The waits are the same functions the kernels use (grid_sync, mbar_wait); the
// probe shows that an expired wait ends the kernel with CESA_ERR_TIMEOUT in the
// control block and leaves the context usable.
#include <cuda_runtime.h>

#include "../../include/cesa.h"
#include "cesa_common.cuh"
#include "cesa_sweep.cuh"

namespace {

constexpr int kWhereGrid = 90;
constexpr int kWhereMbar = 91;

__global__ void wait_probe_kernel(cesa::Ctl* ctl, int which, uint64_t timeout_ns) {
  if (which == 0) {
    // The barrier counts one block more than the launch has, so it never
    // completes; every block gives up after timeout_ns.
    unsigned epoch = 0;
    cesa::grid_sync(ctl, epoch, gridDim.x + 1, timeout_ns, kWhereGrid);
  } else {
    // An mbarrier expecting one arrival that never comes (no copy is issued).
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
      cesa::mbar_init(&bar, 1);
      cesa::mbar_init_fence();
    }
    __syncthreads();
    cesa::mbar_wait(&bar, 0, ctl, timeout_ns, kWhereMbar);
  }
}

__global__ void touch_kernel(int* p) { p[threadIdx.x] += 1; }

}  // namespace

extern "C" int cesa_self_test_waits(int which, int timeout_us, int* status_out, int* where_out) {
  if ((which != 0 && which != 1) || timeout_us < 1 || timeout_us > 10000000 || !status_out || !where_out)
    return CESA_ERR_INVALID_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return CESA_ERR_NO_DEVICE;
  cesa::Ctl* ctl = nullptr;
  if (cudaMalloc(&ctl, sizeof(cesa::Ctl)) != cudaSuccess) return CESA_ERR_OUT_OF_MEMORY;
  int rc = CESA_OK;
  cesa::Ctl h{};
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaFree(ctl);
    return CESA_ERR_CUDA;
  }
  if (cudaMemsetAsync(ctl, 0, sizeof(cesa::Ctl), s) != cudaSuccess) rc = CESA_ERR_CUDA;
  if (rc == CESA_OK) {
    wait_probe_kernel<<<2, 128, 0, s>>>(ctl, which, (uint64_t)timeout_us * 1000ull);
    if (cudaGetLastError() != cudaSuccess) rc = CESA_ERR_CUDA;
  }
  if (rc == CESA_OK && (cudaMemcpyAsync(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                        cudaStreamSynchronize(s) != cudaSuccess))
    rc = CESA_ERR_CUDA;
  // the context must still run work
  if (rc == CESA_OK) {
    int* d = reinterpret_cast<int*>(ctl);
    int v[4] = {0, 0, 0, 0};
    if (cudaMemsetAsync(d, 0, 4 * sizeof(int), s) != cudaSuccess) rc = CESA_ERR_CUDA;
    if (rc == CESA_OK) {
      touch_kernel<<<1, 4, 0, s>>>(d);
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(v, d, sizeof(v), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess || v[0] != 1 || v[3] != 1)
        rc = CESA_ERR_CUDA;
    }
  }
  cudaStreamDestroy(s);
  cudaFree(ctl);
  *status_out = h.status;
  *where_out = h.where;
  return rc;
}

extern "C" int cesa_self_test_partition(int nblk, int nch, int grid, int pair_num, int* kmax_out) {
  if (nblk < 1 || nch < 1 || grid < 1 || pair_num < 0 || pair_num >= cesa::kPairDen || !kmax_out ||
      (pair_num > 0 && (grid & 1)) || (long)nblk * nch > 50000000L)
    return CESA_ERR_INVALID_ARGUMENT;
  cesa::SweepGeom g{};
  g.nblk = nblk;
  g.nch = nch;
  g.ranged = 1;
  g.pair_num = pair_num;
  g.kmax = cesa::ranged_kmax(g, grid);
  *kmax_out = g.kmax;
  long next = 0;
  for (int b = 0; b < grid; ++b) {
    long t0 = 0, t1 = 0;
    cesa::ranged_tasks(g, b, grid, t0, t1);
    if (t0 != next || t1 < t0) return CESA_ERR_INTERNAL;
    next = t1;
    for (long t = t0; t < t1; ++t)
      if (cesa::ranged_block_of(g, t, grid) != b) return CESA_ERR_INTERNAL;
    if (t1 == t0) continue;
    const long o_first = t0 / nch, o_last = (t1 - 1) / nch;
    const int j_first = b - cesa::ranged_block_of(g, o_first * nch, grid);
    if (j_first < 0 || j_first >= g.kmax) return CESA_ERR_INTERNAL;
    for (long o = o_first + 1; o <= o_last; ++o)
      if (cesa::ranged_block_of(g, o * nch, grid) != b) return CESA_ERR_INTERNAL;
  }
  return next == (long)nblk * nch ? CESA_OK : CESA_ERR_INTERNAL;
}
