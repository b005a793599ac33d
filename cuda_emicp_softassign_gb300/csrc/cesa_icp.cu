// ICP for sm_103a: the iterations of icp() (src/icp.cpp:122-290) in one
// persistent cooperative launch.
//
// Reference iteration: every source point y is moved by the current pose,
// z = R y + t, and matched to its nearest target point x_nn; then
//   Xc = mean of the matches, S = sum (x_nn - Xc)(y - Yc)^T (Yc = mean of Y,
//   fixed), pose = findRTfromS(Xc, Yc, S).
// maxIteration iterations, no convergence test. The reference finds the
// matches with FLANN's randomised kd-trees and default search checks, which
// is approximate; here the search is exhaustive (exact nearest neighbour, the
// first of equal distances in X order), tiled over (row block, X slice) units:
//   phase A: a lane owns 4 moved source points (two packed pairs) and scans
//            an X slice staged through shared memory; per element the squared
//            distance by direct differences (3 FADD, FMUL + 2 FFMA, packed)
//            and a compare-select of (distance, index);
//   phase B: after a grid barrier, each row takes the first minimum over the
//            slices in slice order and adds its match to 16 compensated
//            moments (sum x, sum x (y - Yc)^T, sum (y - Yc), sum of distances);
//   after a second barrier every block reduces the moments in a fixed order
//   and solves Horn's pose (the same carried-eigenbasis solve as EM-ICP).
// Coordinates are centred by exact offsets before the loop (S is translation
// invariant; Xc, Yc and t are shifted back).
//
// Grid search (phase A alternative, from 4096 target points on by default):
// the target cloud is bucketed once per registration into a uniform grid of
// about n/4 cells (counting sort: bin, exclusive scan, scatter). A query scans
// the cells in Chebyshev rings around its own cell and stops once the box of
// rings visited is farther from it, on every side, than its best distance
// (with a relative margin for rounding). Candidates are compared on
// (distance, index), so the match is the same as the exhaustive search's and
// the whole registration is bitwise the same. A thread searches its query
// within a work budget; the queries that run over it (far from the target:
// outliers, early misaligned iterations) are searched again after a grid
// barrier by a whole warp each, its lanes splitting every ring's cells. From
// the second iteration on every search starts from the query's previous match
// (a real candidate, so the search stays exact): the pose changes little, so
// the bound starts close to the answer and prunes most cells.
#include <algorithm>

#include "../../include/cesa.h"
#include "cesa_kernels.h"
#include "cesa_ops.cuh"
#include "cesa_pose.h"
#include "cesa_prep.cuh"

namespace cesa {
namespace {

constexpr int kIcpRows = kThreads * 4;  // source points per unit (4 per thread)
constexpr int kIcpTile = 1024;          // target points per shared-memory tile (16 KB)
constexpr int kIcpNV = 16;              // moments: sum x (3), sum x yd^T (9), sum yd (3), sum d2
constexpr int kIcpBudget = 1536;        // per-thread search work (points + 4 x cells) before a warp takes over

// Uniform grid over the (centred) target cloud.
struct IcpGrid {
  float lo[3];  // origin
  float h, inv_h;
  int dim[3];   // cells per axis
  int ncells;
};

// z = R y + t with one fixed rounding (both searches use it, so their squared
// distances agree bit for bit).
__device__ __forceinline__ void move_point(const float (&R)[9], const float (&t)[3], float4 y, float z[3]) {
  for (int i = 0; i < 3; ++i) z[i] = fmaf(R[3 * i], y.x, fmaf(R[3 * i + 1], y.y, fmaf(R[3 * i + 2], y.z, t[i])));
}

__device__ __forceinline__ void consider(float4 q, float zx, float zy, float zz, float& best, int& bi) {
  const float dx = q.x + (-zx), dy = q.y + (-zy), dz = q.z + (-zz);  // as dist2_pair
  float d2 = dx * dx;
  d2 = fmaf(dy, dy, d2);
  d2 = fmaf(dz, dz, d2);
  const int idx = __float_as_int(q.w);
  if (d2 < best || (d2 == best && idx < bi)) {
    best = d2;
    bi = idx;
  }
}

// Scans the points of cell c for the lexicographic minimum of (d2, index),
// four loads in flight.
__device__ __forceinline__ void scan_cell(const int* start, const float4* sorted, int c, float zx, float zy, float zz,
                                          float& best, int& bi) {
  const int e = __ldg(start + c + 1);
  int p = __ldg(start + c);
  for (; p + 4 <= e; p += 4) {
    const float4 q0 = __ldg(sorted + p), q1 = __ldg(sorted + p + 1), q2 = __ldg(sorted + p + 2),
                 q3 = __ldg(sorted + p + 3);
    consider(q0, zx, zy, zz, best, bi);
    consider(q1, zx, zy, zz, best, bi);
    consider(q2, zx, zy, zz, best, bi);
    consider(q3, zx, zy, zz, best, bi);
  }
  for (; p < e; ++p) consider(__ldg(sorted + p), zx, zy, zz, best, bi);
}

// Squared distance (in cell units, a lower bound) from the query at f to cell i;
// cells beyond the best distance are skipped.
__device__ __forceinline__ float cell_gap2(const float (&f)[3], int ix, int iy, int iz) {
  const float gx = fmaxf(fmaxf((float)ix - f[0], f[0] - (float)(ix + 1)), 0.f);
  const float gy = fmaxf(fmaxf((float)iy - f[1], f[1] - (float)(iy + 1)), 0.f);
  const float gz = fmaxf(fmaxf((float)iz - f[2], f[2] - (float)(iz + 1)), 0.f);
  return fmaf(gx, gx, fmaf(gy, gy, gz * gz));
}

// Ring geometry of a query: its position in cell units and its cell.
struct RingQuery {
  float f[3];
  int c[3];
  int r0;  // the first ring that meets the grid
};

__device__ __forceinline__ RingQuery ring_query(const IcpGrid& g, float zx, float zy, float zz) {
  RingQuery q;
  q.f[0] = (zx - g.lo[0]) * g.inv_h;
  q.f[1] = (zy - g.lo[1]) * g.inv_h;
  q.f[2] = (zz - g.lo[2]) * g.inv_h;
  q.r0 = 0;
  for (int a = 0; a < 3; ++a) {
    q.c[a] = (int)floorf(fminf(fmaxf(q.f[a], -1.0e9f), 1.0e9f));
    q.r0 = max(q.r0, max(-q.c[a], q.c[a] - (g.dim[a] - 1)));
  }
  return q;
}

// After ring r: true when every cell has been visited, or when every
// unvisited point (outside the box of cells [c - r, c + r]) is farther than
// the best distance (with relative and absolute margins for rounding).
__device__ __forceinline__ bool ring_done(const IcpGrid& g, const RingQuery& q, int r, float best, bool found) {
  bool whole = true;
  for (int a = 0; a < 3; ++a) whole = whole && q.c[a] - r <= 0 && q.c[a] + r >= g.dim[a] - 1;
  if (whole) return true;
  if (!found) return false;
  float m = 3.0e38f;
  for (int a = 0; a < 3; ++a) m = fminf(m, fminf(q.f[a] - (float)(q.c[a] - r), (float)(q.c[a] + r + 1) - q.f[a]));
  const float bound = fmaxf(m - 1e-4f, 0.f) * g.h;
  return bound * bound > best * (1.f + 1e-5f);
}

// Whether cell i can hold a point nearer than the best distance.
__device__ __forceinline__ bool cell_may_hold(const IcpGrid& g, const RingQuery& q, int ix, int iy, int iz,
                                              float best) {
  const float gap = fmaxf(sqrtf(cell_gap2(q.f, ix, iy, iz)) - 1e-4f, 0.f);
  return gap * gap <= best * (1.f + 1e-5f) * g.inv_h * g.inv_h;
}

// Exact nearest target point of z by rings of cells, one thread. Gives up
// (returns false) once more than `budget` work units (points + 4 x cells)
// have been spent; the query then goes to the warp-cooperative search.
__device__ bool grid_nearest(const IcpGrid& g, const int* start, const float4* sorted, float zx, float zy, float zz,
                             int budget, float seed_d2, int seed_i, float& best_out, int& bi_out) {
  const RingQuery q = ring_query(g, zx, zy, zz);
  float best = seed_d2;  // a real candidate (or +inf and no index)
  int bi = seed_i;
  int work = 0;
  for (int r = q.r0;; ++r) {
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = max(q.c[a] - r, 0);
      hi[a] = min(q.c[a] + r, g.dim[a] - 1);
    }
    for (int ix = lo[0]; ix <= hi[0]; ++ix) {
      const bool bx = ix == q.c[0] - r || ix == q.c[0] + r;
      for (int iy = lo[1]; iy <= hi[1]; ++iy) {
        const bool bxy = bx || iy == q.c[1] - r || iy == q.c[1] + r;
        const int row = (ix * g.dim[1] + iy) * g.dim[2];
        // the shell's cells in this (x, y) column: all of z, or its two z faces
        const int nz = bxy ? hi[2] - lo[2] + 1 : (r > 0 ? 2 : 1);
        for (int k = 0; k < nz; ++k) {
          const int iz = bxy ? lo[2] + k : (k ? q.c[2] + r : q.c[2] - r);
          if (iz < 0 || iz >= g.dim[2]) continue;
          work += 4;
          if (!cell_may_hold(g, q, ix, iy, iz, best)) continue;
          const int cidx = row + iz;
          work += __ldg(start + cidx + 1) - __ldg(start + cidx);
          scan_cell(start, sorted, cidx, zx, zy, zz, best, bi);
        }
        if (work > budget) return false;
      }
    }
    if (ring_done(g, q, r, best, bi != 0x7fffffff)) break;
  }
  best_out = best;
  bi_out = bi;
  return true;
}

// The previous iteration's match as the starting candidate of a search (its
// squared distance computed as the searches compute every candidate's).
__device__ __forceinline__ void seed_of(const float4* cols, const int* prev, int r, int N, float zx, float zy, float zz,
                                        float& d2, int& idx) {
  d2 = __int_as_float(0x7f800000);
  idx = 0x7fffffff;
  const int i = prev ? __ldcg(prev + r) : -1;
  if ((unsigned)i < (unsigned)N) {
    const float4 x = ld_cg(cols + i);
    const float dx = x.x + (-zx), dy = x.y + (-zy), dz = x.z + (-zz);
    float v = dx * dx;
    v = fmaf(dy, dy, v);
    d2 = fmaf(dz, dz, v);
    idx = i;
  }
}

// The same search by a whole warp: each ring's cells are dealt over the lanes,
// each lane keeps its own best, and the lexicographic minimum of (distance,
// index) is reduced over the warp after every ring. All lanes return it.
__device__ void grid_nearest_warp(const IcpGrid& g, const int* start, const float4* sorted, float zx, float zy,
                                  float zz, float seed_d2, int seed_i, float& best_out, int& bi_out) {
  const int lane = threadIdx.x & 31;
  const RingQuery q = ring_query(g, zx, zy, zz);
  float best = seed_d2;
  int bi = seed_i;
  for (int r = q.r0;; ++r) {
    int lo[3], hi[3], n[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = max(q.c[a] - r, 0);
      hi[a] = min(q.c[a] + r, g.dim[a] - 1);
      n[a] = hi[a] - lo[a] + 1;
    }
    const int nbox = n[0] * n[1] * n[2];
    for (int k = lane; k < nbox; k += 32) {
      const int iz = lo[2] + k % n[2];
      const int iy = lo[1] + (k / n[2]) % n[1];
      const int ix = lo[0] + k / (n[2] * n[1]);
      const int cheb = max(max(abs(ix - q.c[0]), abs(iy - q.c[1])), abs(iz - q.c[2]));
      if (cheb != r || !cell_may_hold(g, q, ix, iy, iz, best)) continue;
      scan_cell(start, sorted, (ix * g.dim[1] + iy) * g.dim[2] + iz, zx, zy, zz, best, bi);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (ob < best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (ring_done(g, q, r, best, bi != 0x7fffffff)) break;
  }
  best_out = best;
  bi_out = bi;
}

// One block: the bounding box of the target and the grid (about one cell per
// four target points over the bounding box, at most cap cells).
__global__ void __launch_bounds__(1024) k_icp_grid_setup(const float4* X, int N, int cap, IcpGrid* g) {
  __shared__ float s_lo[3][32], s_hi[3][32];
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const float4 x = X[i];
    const float v[3] = {x.x, x.y, x.z};
    for (int a = 0; a < 3; ++a) {
      lo[a] = fminf(lo[a], v[a]);
      hi[a] = fmaxf(hi[a], v[a]);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int a = 0; a < 3; ++a)
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = fminf(lo[a], __shfl_down_sync(0xffffffffu, lo[a], o));
      hi[a] = fmaxf(hi[a], __shfl_down_sync(0xffffffffu, hi[a], o));
    }
  if (lane == 0)
    for (int a = 0; a < 3; ++a) {
      s_lo[a][warp] = lo[a];
      s_hi[a][warp] = hi[a];
    }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int nw = blockDim.x >> 5;
  double L[3], E[3], emax = 0.0;
  for (int a = 0; a < 3; ++a) {
    float l = s_lo[a][0], h = s_hi[a][0];
    for (int w = 1; w < nw; ++w) {
      l = fminf(l, s_lo[a][w]);
      h = fmaxf(h, s_hi[a][w]);
    }
    L[a] = l;
    E[a] = (double)h - (double)l;
    emax = fmax(emax, E[a]);
  }
  if (!(emax > 0.0)) emax = 1.0;
  for (int a = 0; a < 3; ++a) E[a] = fmax(E[a], 1e-3 * emax);
  const double target = fmax(1.0, fmin((double)cap, N / 4.0));
  double h = cbrt(E[0] * E[1] * E[2] / target);
  int d[3];
  for (int it = 0; it < 64; ++it) {
    long long n = 1;
    for (int a = 0; a < 3; ++a) {
      d[a] = (int)fmin(fmax(ceil(E[a] / h), 1.0), 1024.0);
      n *= d[a];
    }
    if (n <= cap) break;
    h *= 1.1;
  }
  // the cells cover [lo, lo + d h) with a margin of half a cell below
  for (int a = 0; a < 3; ++a) {
    g->lo[a] = (float)(L[a] - 0.5 * h);
    d[a] = min(d[a] + 1, 1024);
  }
  long long n = (long long)d[0] * d[1] * d[2];
  while (n > cap) {  // the margin cell may not fit: drop it on the largest axis
    int a = d[0] >= d[1] && d[0] >= d[2] ? 0 : (d[1] >= d[2] ? 1 : 2);
    d[a] -= 1;
    h *= 1.0 + 1.0 / d[a];
    n = (long long)d[0] * d[1] * d[2];
  }
  g->h = (float)h;
  g->inv_h = (float)(1.0 / h);
  for (int a = 0; a < 3; ++a) g->dim[a] = d[a];
  g->ncells = (int)n;
}

__device__ __forceinline__ int cell_of(const IcpGrid& g, float4 x) {
  int c[3];
  const float v[3] = {x.x, x.y, x.z};
  for (int a = 0; a < 3; ++a) c[a] = min(max((int)floorf((v[a] - g.lo[a]) * g.inv_h), 0), g.dim[a] - 1);
  return (c[0] * g.dim[1] + c[1]) * g.dim[2] + c[2];
}

__global__ void k_icp_bin(const float4* X, int N, const IcpGrid* gp, int* cell, int* count) {
  const IcpGrid g = *gp;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const int c = cell_of(g, X[i]);
    cell[i] = c;
    atomicAdd(count + c, 1);
  }
}

// One block: exclusive scan of the cell counts into start[0..ncells], and a
// copy into the scatter cursors.
__global__ void __launch_bounds__(1024) k_icp_scan(const IcpGrid* gp, const int* count, int* start, int* cursor) {
  __shared__ int s_part[1024];
  const int n = gp->ncells;
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per, e = min(b + per, n);
  int sum = 0;
  for (int i = b; i < e; ++i) sum += count[i];
  s_part[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int k = 0; k < (int)blockDim.x; ++k) {
      const int v = s_part[k];
      s_part[k] = run;
      run += v;
    }
    start[n] = run;
  }
  __syncthreads();
  int run = s_part[threadIdx.x];
  for (int i = b; i < e; ++i) {
    start[i] = run;
    cursor[i] = run;
    run += count[i];
  }
}

// Row order of the source points by the grid cell of their starting position.
__global__ void k_icp_scatter_order(int M, const int* cell, int* cursor, int* order) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x)
    order[atomicAdd(cursor + cell[i], 1)] = i;
}

__global__ void k_icp_scatter(const float4* X, int N, const int* cell, int* cursor, float4* sorted) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const float4 x = X[i];
    const int p = atomicAdd(cursor + cell[i], 1);
    sorted[p] = make_float4(x.x, x.y, x.z, __int_as_float(i));
  }
}

struct IcpArgs {
  const float4* rows;  // Y' centred (M), moved by the pose
  const float4* cols;  // X' centred (N), searched
  int M, N, iters;
  int nrb, S, slice_len, units;
  const CenterHdr* hdr;
  float* dRt;          // PoseIO in/out, caller frame
  float2* part;        // [S][M]: (squared distance, index bits) per slice
  int* nn_out;         // optional [M]: the last iteration's matches
  df* rbpart;          // [2][grid][kIcpNV]
  // grid search (grid != nullptr): cell start offsets [ncells + 1] and the
  // target points sorted by cell, original index in .w
  const IcpGrid* grid;
  const int* cell_start;
  const float4* sorted;
  const int* qorder;   // the rows in the spatial order of their starting position (grid cells)
  int* heavy;          // [M]: rows whose search ran over the per-thread budget
  int* heavy_n;        // their count (reset every iteration)
  int* prev_nn;        // [M]: the previous iteration's matches (grid search's starting candidates)
  Ctl* ctl;
  double* trace;
  int trace_cap;
  int* d_status;
  uint64_t timeout_ns;
};

__global__ void __launch_bounds__(kThreads, 2) icp_kernel(const IcpArgs A) {
  __shared__ float4 s_x[kIcpTile];
  __shared__ float s_pose[12];
  __shared__ float s_hdr[9];  // oX, oY, mean of Y'
  __shared__ df s_red[kThreads];
  __shared__ df s_tot[kIcpNV];
  __shared__ HornState<float> horn;  // carried eigenbasis (thread 0)

  const int tid = threadIdx.x;
  const unsigned G = gridDim.x;
  if (tid == 0) {
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
  unsigned epoch = 0;
  bool ok = true;
  for (int iter = 0; iter < A.iters && ok; ++iter) {
    float R[9], tc[3];
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = s_pose[k];
#pragma unroll
    for (int k = 0; k < 3; ++k) tc[k] = s_pose[9 + k];
    // ---- phase A (grid): each row's nearest point by rings of cells; rows over
    // the per-thread budget are searched again by a whole warp after a barrier
    if (A.grid) {
      const IcpGrid g = *A.grid;
      const int warp = tid >> 5, lane = tid & 31;
      const int nchunks = (A.M + 31) >> 5;
      // warp-sized chunks of spatially ordered rows, dealt round-robin over the blocks
      for (int ch = blockIdx.x + (int)G * warp; ch < nchunks; ch += (int)G * kWarps) {
        const int j = (ch << 5) + lane;
        if (j >= A.M) continue;
        const int r = __ldg(A.qorder + j);
        float z[3];
        move_point(R, tc, ld_cg(A.rows + r), z);
        float best, sd;
        int bi, si;
        seed_of(A.cols, iter > 0 ? A.prev_nn : nullptr, r, A.N, z[0], z[1], z[2], sd, si);
        if (grid_nearest(g, A.cell_start, A.sorted, z[0], z[1], z[2], kIcpBudget, sd, si, best, bi))
          __stcg(A.part + r, make_float2(best, __int_as_float(bi)));
        else
          A.heavy[atomicAdd(A.heavy_n, 1)] = r;
      }
      if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, 69)) {
        ok = false;
        break;
      }
      const int nheavy = ld_acquire(reinterpret_cast<const unsigned*>(A.heavy_n));
      for (int h = blockIdx.x + (int)G * warp; h < nheavy; h += (int)G * kWarps) {
        const int r = __ldcg(A.heavy + h);
        float z[3];
        move_point(R, tc, ld_cg(A.rows + r), z);
        float best, sd;
        int bi, si;
        seed_of(A.cols, iter > 0 ? A.prev_nn : nullptr, r, A.N, z[0], z[1], z[2], sd, si);
        grid_nearest_warp(g, A.cell_start, A.sorted, z[0], z[1], z[2], sd, si, best, bi);
        if (lane == 0) __stcg(A.part + r, make_float2(best, __int_as_float(bi)));
      }
    }
    // ---- phase A (exhaustive): per (row block, X slice), the first nearest point of each row
    for (int u = A.grid ? A.units : blockIdx.x; u < A.units; u += G) {
      const int rb = u / A.S, sl = u - rb * A.S;
      const int cb = sl * A.slice_len, ce = min(cb + A.slice_len, A.N);
      float2 q[2][3];
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        float v[2][3];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          const int r = rb * kIcpRows + (2 * p + l) * kThreads + tid;
          const float4 y = r < A.M ? ld_cg(A.rows + r) : make_float4(0.f, 0.f, 0.f, 0.f);
          float z[3];
          move_point(R, tc, y, z);
          v[l][0] = -z[0];
          v[l][1] = -z[1];
          v[l][2] = -z[2];
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) q[p][d] = make_float2(v[0][d], v[1][d]);
      }
      float bd[2][2];
      int bi[2][2];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          bd[p][l] = __int_as_float(0x7f800000);  // +inf
          bi[p][l] = -1;
        }
      for (int j0 = cb; j0 < ce; j0 += kIcpTile) {
        const int n = min(kIcpTile, ce - j0);
        __syncthreads();
        for (int k = tid; k < n; k += kThreads) s_x[k] = ld_cg(A.cols + j0 + k);
        __syncthreads();
#pragma unroll 8  // independent element chains (exhaustive search 58.5% -> 63.0% of FP32 over 4)
        for (int j = 0; j < n; ++j) {
          const float4 s = s_x[j];
#pragma unroll
          for (int p = 0; p < 2; ++p) {
            const float2 d2 = dist2_pair(q[p], s);
            if (d2.x < bd[p][0]) {
              bd[p][0] = d2.x;
              bi[p][0] = j0 + j;
            }
            if (d2.y < bd[p][1]) {
              bd[p][1] = d2.y;
              bi[p][1] = j0 + j;
            }
          }
        }
      }
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int l = 0; l < 2; ++l) {
          const int r = rb * kIcpRows + (2 * p + l) * kThreads + tid;
          if (r < A.M) __stcg(A.part + (size_t)sl * A.M + r, make_float2(bd[p][l], __int_as_float(bi[p][l])));
        }
    }
    if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, 70)) {
      ok = false;
      break;
    }
    // ---- phase B: the first minimum over the slices, and the moments
    if (A.grid && blockIdx.x == 0 && tid == 0) *A.heavy_n = 0;  // every block is past the heavy rows
    df* mom = A.rbpart + (size_t)(iter & 1) * G * kIcpNV;
    {
      df v[kIcpNV];
#pragma unroll
      for (int k = 0; k < kIcpNV; ++k) v[k] = df_make(0.f);
      for (int r = blockIdx.x * kThreads + tid; r < A.M; r += G * kThreads) {
        float best = __int_as_float(0x7f800000);
        int bi = 0;
        for (int s = 0; s < A.S; ++s) {
          const float2 p = __ldcg(A.part + (size_t)s * A.M + r);
          if (p.x < best) {
            best = p.x;
            bi = __float_as_int(p.y);
          }
        }
        // a source point with a non-finite coordinate matches nothing: no
        // index was recorded, so take the first target point (keeps the read in bounds)
        if ((unsigned)bi >= (unsigned)A.N) bi = 0;
        if (A.nn_out) A.nn_out[r] = bi;
        if (A.prev_nn) __stcg(A.prev_nn + r, bi);  // the next iteration's starting candidate
        const float4 x = ld_cg(A.cols + bi);
        const float4 y = ld_cg(A.rows + r);
        const float xv[3] = {x.x, x.y, x.z};
        const float yd[3] = {y.x - s_hdr[6], y.y - s_hdr[7], y.z - s_hdr[8]};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          df_add(v[i], xv[i]);
          df_add(v[12 + i], yd[i]);
#pragma unroll
          for (int j = 0; j < 3; ++j) df_add_prod(v[3 + i + 3 * j], xv[i], yd[j]);
        }
        df_add(v[15], best);
      }
      block_reduce_df<kIcpNV>(v, s_red);
      if (tid == 0)
#pragma unroll
        for (int k = 0; k < kIcpNV; ++k)
          __stcg(reinterpret_cast<float2*>(mom + (size_t)blockIdx.x * kIcpNV + k), make_float2(v[k].hi, v[k].lo));
    }
    if (!grid_sync(A.ctl, epoch, G, A.timeout_ns, 72)) {
      ok = false;
      break;
    }
    // ---- the pose (every block computes the same one)
    reduce_block_partials<kIcpNV>(mom, (int)G, s_red, s_tot);
    if (tid == 0) {
      float Xc[3], Ym[3], S[9];
      for (int i = 0; i < 3; ++i) {
        Xc[i] = (float)(df_dbl(s_tot[i]) / (double)A.M);
        Ym[i] = s_hdr[6 + i];
      }
      // S = sum (x - Xc)(y - Yc)^T = sum x yd^T - Xc (sum yd)^T
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          df a = s_tot[3 + i + 3 * j];
          df_add_prod(a, -Xc[i], df_val(s_tot[12 + j]));
          S[i + 3 * j] = df_val(a);
        }
      float q[4], gap = 0.f, lmax = 0.f, Rn[9], tn[3];
      horn_quaternion_fast<float>(S, horn, q, &gap, &lmax);
      quat_to_pose<float>(q, Xc, Ym, Rn, tn);  // centred frame: t' = Xc' - R Ym
      for (int k = 0; k < 9; ++k) s_pose[k] = Rn[k];
      for (int k = 0; k < 3; ++k) s_pose[9 + k] = tn[k];
      if (blockIdx.x == 0) {
        if (A.trace && iter < A.trace_cap) {
          double* rec = A.trace + (size_t)iter * 32;
          float to[3];
          pose_from_centred(Rn, tn, &s_hdr[0], &s_hdr[3], to);
          rec[0] = iter;
          rec[1] = iter;
          rec[2] = df_dbl(s_tot[15]);
          for (int i = 0; i < 3; ++i) {
            rec[3 + i] = (double)Xc[i] + s_hdr[i];
            rec[6 + i] = (double)Ym[i] + s_hdr[3 + i];
            rec[27 + i] = to[i];
          }
          for (int k = 0; k < 9; ++k) {
            rec[9 + k] = S[k];
            rec[18 + k] = Rn[k];
          }
          rec[30] = gap;
          rec[31] = lmax;
        }
        A.ctl->steps_done = iter + 1;
      }
    }
    __syncthreads();
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

struct IcpPlan {
  int grid, nrb, S, slice_len, units;
  bool use_grid;
  int cap;  // cells at most
};

// Row blocks of kIcpRows source points and X slices of at least 256 points,
// as many slices as fill whole waves of the co-resident grid best (up to 4).
IcpPlan plan_icp(int N, int M, int device, int search) {
  IcpPlan P;
  const int limit = persistent_grid_limit(device, (const void*)icp_kernel, 0);
  P.use_grid = search == CESA_ICP_SEARCH_GRID || (search == CESA_ICP_SEARCH_AUTO && N >= 4096);
  P.cap = std::max(64, N / 4);
  if (P.use_grid) {  // one slice: every row is searched whole by one thread
    P.nrb = (M + kIcpRows - 1) / kIcpRows;
    P.S = 1;
    P.slice_len = N;
    P.units = 0;
    P.grid = limit;  // rows are dealt in warp-sized chunks over all co-resident blocks
    return P;
  }
  P.nrb = (M + kIcpRows - 1) / kIcpRows;
  const int max_s = (N + 255) / 256;
  int bestS = 1;
  double best = -1.0;
  for (int w = 1; w <= 4; ++w) {
    int S = (w * limit) / P.nrb;
    if (S < 1) S = 1;
    if (S > max_s) S = max_s;
    const int units = P.nrb * S;
    const int waves = (units + limit - 1) / limit;
    const double eff = (double)units / ((double)waves * limit);
    if (eff > best + 0.02) {
      best = eff;
      bestS = S;
    }
  }
  P.slice_len = (N + bestS - 1) / bestS;
  P.S = (N + P.slice_len - 1) / P.slice_len;
  P.units = P.nrb * P.S;
  P.grid = P.units < limit ? P.units : limit;
  return P;
}

struct IcpCarved {
  Ctl* ctl;
  CenterHdr* hdr;
  float4* rows;
  float4* cols;
  float2* part;
  df* rbpart;
  IcpGrid* grid;  // grid search only
  int *count, *start, *cursor, *cell;
  float4* sorted;
  int* qorder;
  int* heavy;
  int* heavy_n;
  int* prev_nn;
};

IcpCarved carve_icp(void* base, const IcpPlan& P, int N, int M, size_t* total) {
  Carve c(base);
  IcpCarved w{};
  w.ctl = c.take<Ctl>(1);
  w.hdr = c.take<CenterHdr>(1);
  w.rows = c.take<float4>((size_t)M);
  w.cols = c.take<float4>((size_t)N);
  w.part = c.take<float2>((size_t)P.S * M);
  w.rbpart = c.take<df>((size_t)2 * P.grid * kIcpNV);
  if (P.use_grid) {
    w.grid = c.take<IcpGrid>(1);
    w.count = c.take<int>((size_t)P.cap + 1);
    w.start = c.take<int>((size_t)P.cap + 1);
    w.cursor = c.take<int>((size_t)P.cap + 1);
    w.cell = c.take<int>((size_t)std::max(N, M));
    w.sorted = c.take<float4>((size_t)N);
    w.qorder = c.take<int>((size_t)M);
    w.heavy = c.take<int>((size_t)M);
    w.heavy_n = c.take<int>(1);
    w.prev_nn = c.take<int>((size_t)M);
  }
  if (total) *total = c.off;
  return w;
}

}  // namespace

size_t icp_ws_need(int N, int M, int device, int search) {
  const IcpPlan P = plan_icp(N, M, device, search);
  size_t total = 0;
  carve_icp(nullptr, P, N, M, &total);
  return total;
}

int enqueue_icp(const IcpLaunch& L, void* ws, size_t ws_bytes, cudaStream_t st, int* grid_used) {
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return (int)e;
  const IcpPlan P = plan_icp(L.N, L.M, device, L.search);
  size_t total = 0;
  IcpCarved w = carve_icp(ws, P, L.N, L.M, &total);
  if (total > ws_bytes) return (int)cudaErrorInvalidValue;
  if (grid_used) *grid_used = P.grid;
  e = cudaMemsetAsync(w.ctl, 0, sizeof(Ctl), st);
  if (e != cudaSuccess) return (int)e;
  prep_center_kernel<<<1, 1024, 0, st>>>(L.dX, L.N, L.dY, L.M, w.hdr);
  const int pb = 256, pg_x = (L.N + pb - 1) / pb, pg_y = (L.M + pb - 1) / pb;
  prep_pack_kernel<<<pg_x < 1024 ? pg_x : 1024, pb, 0, st>>>(L.dX, L.N, w.hdr, 0, 0.f, w.cols);
  prep_pack_kernel<<<pg_y < 1024 ? pg_y : 1024, pb, 0, st>>>(L.dY, L.M, w.hdr, 1, 0.f, w.rows);
  if (P.use_grid) {  // bucket the target once for all iterations
    e = cudaMemsetAsync(w.heavy_n, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.count, 0, sizeof(int) * ((size_t)P.cap + 1), st);
    if (e != cudaSuccess) return (int)e;
    k_icp_grid_setup<<<1, 1024, 0, st>>>(w.cols, L.N, P.cap, w.grid);
    const int gb = std::min((L.N + pb - 1) / pb, 1024);
    k_icp_bin<<<gb, pb, 0, st>>>(w.cols, L.N, w.grid, w.cell, w.count);
    k_icp_scan<<<1, 1024, 0, st>>>(w.grid, w.count, w.start, w.cursor);
    k_icp_scatter<<<gb, pb, 0, st>>>(w.cols, L.N, w.cell, w.cursor, w.sorted);
    // the source rows in the spatial order of their starting positions (a rigid
    // motion keeps neighbours together, so a warp's queries stay coherent)
    e = cudaMemsetAsync(w.count, 0, sizeof(int) * ((size_t)P.cap + 1), st);
    if (e != cudaSuccess) return (int)e;
    const int gy = std::min((L.M + pb - 1) / pb, 1024);
    k_icp_bin<<<gy, pb, 0, st>>>(w.rows, L.M, w.grid, w.cell, w.count);
    k_icp_scan<<<1, 1024, 0, st>>>(w.grid, w.count, w.cursor, w.cursor);
    k_icp_scatter_order<<<gy, pb, 0, st>>>(L.M, w.cell, w.cursor, w.qorder);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (L.iters <= 0) return 0;
  IcpArgs A;
  A.rows = w.rows;
  A.cols = w.cols;
  A.M = L.M;
  A.N = L.N;
  A.iters = L.iters;
  A.nrb = P.nrb;
  A.S = P.S;
  A.slice_len = P.slice_len;
  A.units = P.units;
  A.hdr = w.hdr;
  A.dRt = L.dRt;
  A.part = w.part;
  A.nn_out = L.nn_out;
  A.rbpart = w.rbpart;
  A.grid = P.use_grid ? w.grid : nullptr;
  A.cell_start = w.start;
  A.sorted = w.sorted;
  A.qorder = w.qorder;
  A.heavy = w.heavy;
  A.heavy_n = w.heavy_n;
  A.prev_nn = P.use_grid ? w.prev_nn : nullptr;
  A.ctl = w.ctl;
  A.trace = L.trace;
  A.trace_cap = L.trace_cap;
  A.d_status = L.d_status;
  A.timeout_ns = L.timeout_ns;
  void* args[] = {(void*)&A};
  return (int)cudaLaunchCooperativeKernel((const void*)icp_kernel, dim3(P.grid), dim3(kThreads), args, 0, st);
}

}  // namespace cesa
