/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * Host runtime of cuda_emu.h: device memory, kernel launches (one fiber per
 * CUDA thread, ucontext), the block barrier, and the legacy cuBLAS calls over
 * Fortran BLAS.
 */
#include <stdlib.h>
#include <string.h>
#include <ucontext.h>

#include <vector>

#include "cublas.h"
#include "cuda_emu.h"

// ---------------------------------------------------------------- memory
namespace {
constexpr size_t kPad = 4096;  // slack after every buffer (see cuda_emu.h)
}

cudaError_t cudaMalloc(void** p, size_t bytes) {
  *p = calloc(1, bytes + kPad);
  return *p ? cudaSuccess : 2;
}
cudaError_t cudaFree(void* p) {
  free(p);
  return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, cudaMemcpyKind) {
  memmove(dst, src, bytes);
  return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
cudaError_t cudaDeviceReset() { return cudaSuccess; }
cudaError_t cudaThreadSynchronize() { return cudaSuccess; }
cudaError_t cudaThreadExit() { return cudaSuccess; }

// ---------------------------------------------------------------- launches
namespace cesa_emu {

thread_local dim3 g_block_idx;
thread_local dim3 g_block_dim;
thread_local dim3 g_grid_dim;
thread_local dim3* g_thread_idx = nullptr;

namespace {

enum State { kReady, kParked, kDone };
constexpr size_t kStack = 32 * 1024;

// The fibers of the block running on this host thread.
struct Block {
  std::vector<ucontext_t> ctx;
  std::vector<char> stacks;
  std::vector<int> state;
  std::vector<dim3> tid;
  ucontext_t sched;
  int cur = 0;
  const std::function<void()>* body = nullptr;
};

thread_local Block* t_block = nullptr;
thread_local Block t_fibers;  // kept across launches: the stacks are allocated once per host thread

void fiber_main() {
  Block* b = t_block;
  (*b->body)();
  b->state[b->cur] = kDone;
  // returning resumes b->sched (uc_link)
}

void run_block(Block& b, const dim3& blk, const std::function<void()>& body) {
  const int n = (int)(blk.x * blk.y * blk.z);
  if ((int)b.ctx.size() < n) {
    b.ctx.resize(n);
    b.stacks.resize((size_t)n * kStack);
    b.state.resize(n);
    b.tid.resize(n);
  }
  b.body = &body;
  for (int i = 0; i < n; ++i) {
    b.tid[i] = dim3(i % blk.x, (i / blk.x) % blk.y, i / (blk.x * blk.y));
    getcontext(&b.ctx[i]);
    b.ctx[i].uc_stack.ss_sp = b.stacks.data() + (size_t)i * kStack;
    b.ctx[i].uc_stack.ss_size = kStack;
    b.ctx[i].uc_link = &b.sched;
    makecontext(&b.ctx[i], fiber_main, 0);
    b.state[i] = kReady;
  }
  for (;;) {
    // run every ready fiber until it parks at the barrier or returns
    for (int i = 0; i < n; ++i) {
      if (b.state[i] != kReady) continue;
      b.cur = i;
      g_thread_idx = &b.tid[i];
      swapcontext(&b.sched, &b.ctx[i]);
    }
    int parked = 0;
    for (int i = 0; i < n; ++i) parked += b.state[i] == kParked;
    if (!parked) break;
    // every fiber still running is parked: the barrier opens
    for (int i = 0; i < n; ++i)
      if (b.state[i] == kParked) b.state[i] = kReady;
  }
  g_thread_idx = nullptr;
}

}  // namespace

void syncthreads() {
  Block* b = t_block;
  const int i = b->cur;
  b->state[i] = kParked;
  swapcontext(&b->ctx[i], &b->sched);
}

void Launch::run(const std::function<void()>& body) const {
  const long nblocks = (long)grid.x * grid.y * grid.z;
  const dim3 g = grid, blk = block;
#pragma omp parallel
  {
    Block& b = t_fibers;
    t_block = &b;
    g_grid_dim = g;
    g_block_dim = blk;
#pragma omp for schedule(dynamic, 4)
    for (long k = 0; k < nblocks; ++k) {
      g_block_idx = dim3((unsigned)(k % g.x), (unsigned)((k / g.x) % g.y), (unsigned)(k / ((long)g.x * g.y)));
      run_block(b, blk, body);
    }
    t_block = nullptr;
  }
}

}  // namespace cesa_emu

// ---------------------------------------------------------------- cuBLAS
extern "C" {
int sgemv_(const char*, const int*, const int*, const float*, const float*, const int*, const float*, const int*,
           const float*, float*, const int*);
int saxpy_(const int*, const float*, const float*, const int*, float*, const int*);
float sasum_(const int*, const float*, const int*);
int sscal_(const int*, const float*, float*, const int*);
int sgemm_(const char*, const char*, const int*, const int*, const int*, const float*, const float*, const int*,
           const float*, const int*, const float*, float*, const int*);
}

cublasStatus cublasInit() { return 0; }
cublasStatus cublasShutdown() { return 0; }

void cublasSgemv(char trans, int m, int n, float alpha, const float* A, int lda, const float* x, int incx,
                 float beta, float* y, int incy) {
  sgemv_(&trans, &m, &n, &alpha, A, &lda, x, &incx, &beta, y, &incy);
}
void cublasSaxpy(int n, float alpha, const float* x, int incx, float* y, int incy) {
  saxpy_(&n, &alpha, x, &incx, y, &incy);
}
float cublasSasum(int n, const float* x, int incx) { return sasum_(&n, x, &incx); }
void cublasSscal(int n, float alpha, float* x, int incx) { sscal_(&n, &alpha, x, &incx); }
void cublasSgemm(char transa, char transb, int m, int n, int k, float alpha, const float* A, int lda,
                 const float* B, int ldb, float beta, float* C, int ldc) {
  sgemm_(&transa, &transb, &m, &n, &k, &alpha, A, &lda, B, &ldb, &beta, C, &ldc);
}
