// Throughput probes for the roofline denominators of the registration
// kernels (built into libcesa_peaks.so, used by bench.py). The kernels here
// are FP32-pipe / MUFU-bound, and the measured-peak file of the machine only
// carries HBM copy bandwidth and tensor-core GEMM rates, so the FP32 FFMA and
// MUFU ex2 rates are measured on the same GPU in the same run.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

__global__ void ffma_rate_kernel(float* out, int iters, float a) {
  float x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fmaf(x[i], a, 0.5f);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void ex2_rate_kernel(float* out, int iters) {
  float x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = 0.3f + 0.01f * i + threadIdx.x * 1e-5f;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float y;
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-x[i]));
      x[i] = y;
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class F>
double timed_rate(F launch, double ops, int reps) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();  // warm-up
  cudaDeviceSynchronize();
  float best = 1e30f;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ops / (best * 1e-3);
}

}  // namespace

extern "C" {

// FP32 FFMA lane-operations per second (one FMA = 1 op) and MUFU ex2
// operations per second on the current device; 0 on success.
int cesa_peaks_measure(double* fp32_ops_per_s, double* ex2_ops_per_s) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8, iters = 8192;
  float* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(float) * (size_t)blocks * threads) != cudaSuccess) return 2;
  const double n = (double)blocks * threads * iters * 8.0;
  *fp32_ops_per_s = timed_rate([&] { ffma_rate_kernel<<<blocks, threads>>>(buf, iters, 0.999f); }, n, 5);
  *ex2_ops_per_s = timed_rate([&] { ex2_rate_kernel<<<blocks, threads>>>(buf, iters / 4); }, n / 4, 5);
  const cudaError_t e = cudaGetLastError();
  cudaFree(buf);
  return e == cudaSuccess ? 0 : 3;
}

}  // extern "C"
