/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- never linked into the product.
 *
 * A CPU emulation of the small part of the CUDA runtime that the reference's
 * GPU sources use (src/softassign.cu, src/emicp.cu), so that their own code
 * runs on the host as a checker where no GPU may run it (their kernels call
 * __syncthreads() inside divergent branches, and one reads past its input;
 * neither is run on a shared GPU).
 *
 * oracle/build.py compiles such a source with g++ and `-include cuda_emu.h`.
 * The one change to the source is mechanical: every launch
 *     kernel <<< grid, block >>> (args);
 * becomes
 *     cesa_emu::Launch(grid, block).run([&] { kernel(args); });
 * Everything else compiles as written:
 *   - __global__, __device__, __host__ vanish; __shared__ becomes a
 *     function-static, thread_local array (one block runs at a time on each
 *     host thread, so it is the block's shared memory);
 *   - every CUDA thread of a block is a fiber (ucontext) on one host thread;
 *     __syncthreads() parks the fiber until every fiber of the block that has
 *     not returned is parked, as a block barrier does (threads that leave the
 *     kernel no longer take part);
 *   - the blocks of a grid run in parallel over OpenMP threads, each with its
 *     own fibers (the kernels share nothing across blocks);
 *   - device memory is host memory (cudaMalloc pads every buffer by 4 KiB and
 *     zero-fills it, so the reference's read past an input stays inside it);
 *   - the legacy cuBLAS calls go to Fortran BLAS (cublas.h in this directory).
 */
#ifndef CESA_CUDA_EMU_H_
#define CESA_CUDA_EMU_H_

#include <cmath>
#include <cstddef>
#include <functional>

struct dim3 {
  unsigned x, y, z;
  dim3(unsigned x_ = 1, unsigned y_ = 1, unsigned z_ = 1) : x(x_), y(y_), z(z_) {}
};

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3,
  cudaMemcpyDefault = 4
};

cudaError_t cudaMalloc(void** p, size_t bytes);
cudaError_t cudaFree(void* p);
cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind);
cudaError_t cudaDeviceSynchronize();
cudaError_t cudaDeviceReset();
cudaError_t cudaThreadSynchronize();
cudaError_t cudaThreadExit();

namespace cesa_emu {

extern thread_local dim3 g_block_idx;
extern thread_local dim3 g_block_dim;
extern thread_local dim3 g_grid_dim;
extern thread_local dim3* g_thread_idx;

void syncthreads();

// Runs `body` once per CUDA thread of every block of the grid.
struct Launch {
  dim3 grid, block;
  Launch(dim3 g, dim3 b) : grid(g), block(b) {}
  void run(const std::function<void()>& body) const;
};

}  // namespace cesa_emu

#define __global__
#define __device__
#define __host__
#define __shared__ static thread_local
#define __syncthreads() cesa_emu::syncthreads()
#define threadIdx (*cesa_emu::g_thread_idx)
#define blockIdx (cesa_emu::g_block_idx)
#define blockDim (cesa_emu::g_block_dim)
#define gridDim (cesa_emu::g_grid_dim)

#endif
