// Device utilities shared by the registration kernels (sm_103a).
//
//  * ex2.approx on the MUFU pipe (the only transcendental in the hot loops);
//  * double-float ("df") compensated sums on the FP32 pipe. GB300 executes
//    FP64 at ~1.7 DFMA/clk/SM with ~64-cycle dependent latency, so every
//    cross-row and cross-block reduction is kept in (hi, lo) float pairs
//    (TwoSum / TwoProd, ~48-bit significand) instead of FP64;
//  * a bounded grid barrier for the persistent cooperative kernels;
//  * 1-D TMA bulk copies (cp.async.bulk) completed on an mbarrier, with
//    bounded waits.
// Every wait has a time limit. On expiry the block records CESA_ERR_TIMEOUT in
// the control block and returns, so the host reads an error status instead of
// a hung context.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cesa {

constexpr int kStatusOk = 0;
constexpr int kStatusTimeout = 3;      // == CESA_ERR_TIMEOUT
constexpr int kStatusUnsupported = 6;  // == CESA_ERR_UNSUPPORTED (a launch shape the kernel cannot run)
constexpr int kStatusInternal = 8;     // == CESA_ERR_INTERNAL (an index check failed; the access was skipped)

constexpr float kLog2e = 1.4426950408889634f;

// Control block in device memory, zeroed before each persistent launch.
struct Ctl {
  unsigned bar;      // grid-barrier arrival counter (monotonic)
  int status;        // first error recorded by any block
  int where;         // which wait gave up (diagnostic)
  int steps_done;    // pose updates completed
  unsigned pad[12];
};

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ int ld_status(const Ctl* ctl) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(&ctl->status) : "memory");
  return v;
}

__device__ __forceinline__ void set_status(Ctl* ctl, int code, int where) {
  if (atomicCAS(&ctl->status, 0, code) == 0) ctl->where = where;
}

// Optional phase timeline, recorded by thread 0 of every block into its own
// region of cap / gridDim.x entries.
struct Timeline {
  unsigned long long* p;
  int cap;
  int n;
  __device__ __forceinline__ void mark(int phase) {
    const int per = cap / (int)gridDim.x;
    if (p && threadIdx.x == 0 && n < per)
      p[(size_t)blockIdx.x * per + n++] = ((unsigned long long)phase << 56) | (global_ns() & ((1ull << 56) - 1));
  }
};

// ---------------------------------------------------------------- double-float
struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float v) { return df{v, 0.f}; }

// a += b (TwoSum; error term folded into lo). The _rn intrinsics keep the
// compiler from contracting or reassociating the compensated arithmetic.
__device__ __forceinline__ void df_add(df& a, float b) {
  float s = __fadd_rn(a.hi, b);
  float bb = __fsub_rn(s, a.hi);
  float err = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  a.hi = s;
  a.lo = __fadd_rn(a.lo, err);
}

// a += x*y exactly up to the df precision (TwoProd via FMA).
__device__ __forceinline__ void df_add_prod(df& a, float x, float y) {
  float p = __fmul_rn(x, y);
  float e = __fmaf_rn(x, y, -p);
  df_add(a, p);
  a.lo = __fadd_rn(a.lo, e);
}

__device__ __forceinline__ void df_add(df& a, const df& b) {
  df_add(a, b.hi);
  a.lo = __fadd_rn(a.lo, b.lo);
}

__device__ __forceinline__ float df_val(const df& a) { return __fadd_rn(a.hi, a.lo); }
__device__ __forceinline__ double df_dbl(const df& a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df df_shfl_down(const df& a, int off) {
  return df{__shfl_down_sync(0xffffffffu, a.hi, off), __shfl_down_sync(0xffffffffu, a.lo, off)};
}

// Sum of NV df values over the block (blockDim.x threads, multiple of 32).
// red: shared scratch of NV * (blockDim.x/32) dfs. Result valid in thread 0.
// Fixed reduction order, so the result is bitwise reproducible.
template <int NV>
__device__ __forceinline__ void block_reduce_df(df (&v)[NV], df* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      df o = df_shfl_down(v[k], off);
      df_add(v[k], o);
    }
  }
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) red[k * nw + warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      df s = red[k * nw];
      for (int w = 1; w < nw; ++w) df_add(s, red[k * nw + w]);
      v[k] = s;
    }
  }
}

// ---------------------------------------------------------------- grid barrier
// Release add (no return value): orders this thread's earlier writes, and the
// block's writes it observed through __syncthreads, before the add.
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Acquire-release add returning the old value.
__device__ __forceinline__ unsigned atom_acq_rel_add(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Monotonic-counter barrier over `nblocks` blocks of a cooperative launch that
// share the counter `bar` (every block of the grid, or a fixed group of them).
// `epoch` counts the barriers this block has passed on that counter (kept by
// the caller). Thread 0 arrives with a release add and polls with acquire
// loads; the __syncthreads on either side extend the ordering to the whole
// block. Returns false when the wait exceeded timeout_ns or another block
// recorded an error while this one waited; the caller must then leave the
// kernel, or skip its work while still meeting its cluster barriers.
__device__ __forceinline__ bool counter_sync(unsigned* bar, Ctl* ctl, unsigned& epoch, unsigned nblocks,
                                             uint64_t timeout_ns, int where) {
  __shared__ int s_ok;
  __syncthreads();
  epoch += 1;
  if (threadIdx.x == 0) {
    const unsigned target = epoch * nblocks;
    red_release_add(bar, 1u);
    int ok = 1;
    uint64_t t0 = 0;
    unsigned spins = 0;
    while ((int)(ld_acquire(bar) - target) < 0) {
      if ((++spins & 31u) == 0) {
        if (ld_status(ctl) != kStatusOk) {
          ok = 0;
          break;
        }
        const uint64_t now = global_ns();
        if (t0 == 0) {
          t0 = now;
        } else if (now - t0 > timeout_ns) {
          set_status(ctl, kStatusTimeout, where);
          ok = 0;
          break;
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The barrier across all blocks of the launch.
__device__ __forceinline__ bool grid_sync(Ctl* ctl, unsigned& epoch, unsigned nblocks,
                                          uint64_t timeout_ns, int where) {
  return counter_sync(&ctl->bar, ctl, epoch, nblocks, timeout_ns, where);
}

// ---------------------------------------------------------------- clusters
// Barrier over all threads of every CTA of the thread-block cluster (every
// thread must call it, convergently): release of this CTA's prior writes,
// acquire of the peers'. It has no time limit, so a kernel calls it the same
// number of times in every CTA of a cluster, whatever happens elsewhere.
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_ctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned cluster_nctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned cluster_id_x() {
  unsigned r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}

// Shared-memory address of `p` (a variable of this CTA's shared memory) in the
// CTA of cluster rank `rank`.
__device__ __forceinline__ uint32_t dsmem_addr(const void* p, unsigned rank) {
  const uint32_t a = static_cast<uint32_t>(__cvta_generic_to_shared(p));
  uint32_t b;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(b) : "r"(a), "r"(rank));
  return b;
}

__device__ __forceinline__ float ld_dsmem(const float* p, unsigned rank) {
  float v;
  asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(dsmem_addr(p, rank)) : "memory");
  return v;
}

__device__ __forceinline__ df ld_dsmem(const df* p, unsigned rank) {
  df v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.hi), "=f"(v.lo) : "r"(dsmem_addr(p, rank)) : "memory");
  return v;
}

// ---------------------------------------------------------------- TMA bulk copy
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Global -> shared bulk copy (bytes % 16 == 0, both addresses 16-byte aligned),
// completion counted on `bar` as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Bounded wait for phase `parity` of `bar`. On expiry records the timeout,
// then waits once more (bounded) so that a copy still in flight lands before
// the block leaves; returns false if the phase never completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, Ctl* ctl,
                                          uint64_t timeout_ns, int where) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > timeout_ns) break;
  }
  set_status(ctl, kStatusTimeout, where);
  const uint64_t t1 = global_ns();
  while (global_ns() - t1 < timeout_ns) {
    if (mbar_try_wait(bar, parity)) break;
  }
  return false;
}

// L2-coherent loads for data written by other blocks during the same launch.
__device__ __forceinline__ float4 ld_cg(const float4* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_cg(const float* p) { return __ldcg(p); }

}  // namespace cesa
