/*
 * cesa.h -- C ABI of the GB300-native soft-correspondence registration library
 * (libcesa.so): annealed EM-ICP and Softassign (and plain ICP) rigid
 * registration on one GPU.
 *
 * Every entry point takes plain pointers and sizes. Point sets are SoA float
 * arrays [x0..xn-1, y0..yn-1, z0..zn-1], the layout the reference builds with
 * cloud2data() (src/cloud2data.cpp:29-46). The rotation R is 9 floats,
 * row-major (r11 r12 r13 r21 ...), and t is 3 floats (README.md:205-214). On
 * entry R,t is the initial pose; on exit it is the estimate such that
 * X ~ R*Y + t (X = target, Y = source).
 *
 * All functions return CESA_OK (0) or a CESA_ERR_* code; nothing calls exit().
 * The reference's functions return void and ignore CUDA errors
 * (src/3dregistration.h:118); the C++ drop-in layer (3dregistration.h in this
 * directory) keeps void and reports failures on stderr.
 */
#ifndef CESA_H_
#define CESA_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CESA_OK 0
#define CESA_ERR_INVALID_ARGUMENT 1 /* bad size, NULL pointer, bad parameter */
#define CESA_ERR_CUDA 2             /* a CUDA runtime call failed */
#define CESA_ERR_TIMEOUT 3          /* a device-side wait gave up after its limit */
#define CESA_ERR_NO_DEVICE 4        /* no usable CUDA device */
#define CESA_ERR_OUT_OF_MEMORY 5    /* device or host allocation failed */
#define CESA_ERR_UNSUPPORTED 6      /* the request is outside what this build supports */
#define CESA_ERR_NOALLOC_LIMIT 7    /* too large for the fixed scratch of cesa_emicp_device_noalloc */
#define CESA_ERR_INTERNAL 8         /* a kernel's own consistency check failed (a bug; the access was skipped) */

/* cudaStream_t without including cuda_runtime.h (same underlying type). */
typedef struct CUstream_st* cesa_stream_t;

/* Sinkhorn normalisation forms for Softassign (cesa_params.sinkhorn_form). */
#define CESA_SINKHORN_AUTO 0         /* per-size choice by the built-in tuner */
#define CESA_SINKHORN_MATRIX_FREE 1  /* scaling vectors, affinities recomputed per sweep */
#define CESA_SINKHORN_MATERIALISED 2 /* affinity matrix stored once per inner iteration */
#define CESA_SINKHORN_BANDED 3       /* matrix-free, one thread-block cluster per band of 64 rows
                                        (M <= 2048 and all bands resident; else the matrix-free form) */

/* Work decomposition of the EM-ICP backward's sweep (cesa_params.emicp_backward_layout).
   Every layout computes the same gradient; they differ in the summation order of
   the partial sums (each deterministic) and in speed. */
#define CESA_LAYOUT_AUTO 0    /* by size: ranged where its longest task run is the shorter */
#define CESA_LAYOUT_SLICES 1  /* units of (1536 X columns, slice of Y rows) dealt round-robin */
#define CESA_LAYOUT_RANGED 2  /* each block a contiguous run of (1536 columns, 256 rows) tasks */

/* Execution of the Softassign backward (cesa_params.softassign_backward_form).
   Both compute the same gradient up to the summation order of partial sums. */
#define CESA_SA_BACKWARD_AUTO 0       /* by size: persistent up to N x M = 16e6, else per-update launches */
#define CESA_SA_BACKWARD_PERSISTENT 1 /* one cooperative launch over all updates (the launches where it cannot) */
#define CESA_SA_BACKWARD_LAUNCHES 2   /* each update's launch sequence, replayed as a CUDA graph */

/*
 * Registration parameters. The first twelve fields mirror
 * registrationParameters (src/3dregistration.h:39-57) in name, type, order and
 * meaning. The remaining fields control the GPU path and have no counterpart
 * in the reference. cesa_params_default() fills the reference CLI defaults
 * (src/main.cpp:280-315).
 */
typedef struct cesa_params {
  /* Softassign */
  int JMAX;        /* annealing steps; T <- T*TFACTOR after each */
  int I0;          /* pose updates per temperature */
  int I1;          /* Sinkhorn row/column passes per pose update (>= 1) */
  float alpha;     /* outlier parameter */
  float T_0;       /* initial temperature */
  float TFACTOR;   /* temperature factor */
  float moutlier;  /* initial slack-row / slack-column value */
  /* EM-ICP */
  float sigma_p2;     /* initial sigma_p^2; sigma_p2 <- sigma_p2*sigma_factor while > sigma_inf */
  float sigma_inf;    /* stop value of sigma_p2 */
  float sigma_factor; /* factor for sigma_p2 */
  float d_02;         /* outlier distance^2 */
  /* ICP */
  int maxIteration;   /* iterations of cesa_icp (no convergence test, as the reference) */
  /* GPU path controls */
  int sinkhorn_form; /* CESA_SINKHORN_* */
  int timeout_ms;    /* limit of any device-side wait; 0 selects 10000 ms */
  int device;        /* CUDA device ordinal for the host-pointer entry points; -1 = current */
  int icp_search;    /* CESA_ICP_SEARCH_*: nearest-neighbour search of cesa_icp */
  int emicp_backward_layout;   /* CESA_LAYOUT_*: work decomposition of cesa_emicp_backward_device */
  int softassign_backward_form; /* CESA_SA_BACKWARD_*: execution of cesa_softassign_backward_device */
  int reserved[2];
} cesa_params;

/* ICP nearest-neighbour search (cesa_params.icp_search). Both are exact and
 * give the same matches (the first of equal distances in X order). */
#define CESA_ICP_SEARCH_AUTO 0       /* uniform grid from 4096 target points on, else exhaustive */
#define CESA_ICP_SEARCH_EXHAUSTIVE 1 /* every target point, tiled through shared memory */
#define CESA_ICP_SEARCH_GRID 2       /* uniform grid over the target, rings of cells around each query */

/*
 * Optional per-call report (may be NULL). trace, when non-NULL, receives one
 * record of CESA_TRACE_STRIDE doubles per pose update, up to trace_capacity:
 *   [0] step  [1] sigma_p2 or T  [2] sum(lambda) or sumM  [3..5] Xc  [6..8] Yc
 *   [9..17] S (reference h_S layout, S[i+3j])  [18..26] R row-major  [27..29] t
 *   [30] relative eigen-gap of Horn's N  [31] largest eigenvalue of N
 */
#define CESA_TRACE_STRIDE 32
typedef struct cesa_report {
  double* trace;        /* host buffer or NULL */
  int trace_capacity;   /* records */
  int steps;            /* out: pose updates performed */
  int sinkhorn_form;    /* out: form used (Softassign) */
  int grid_blocks;      /* out: persistent grid size */
  float device_ms;      /* out: device time of the registration kernels */
  /* Optional phase timeline (profiling): block b of the persistent grid
   * records into entries [b * per, (b + 1) * per), per = timeline_capacity /
   * grid_blocks; an entry is (phase << 56) | (globaltimer ns & (2^56 - 1)),
   * 0 when unused. Phases are listed in CESA_TL_* below. */
  unsigned long long* timeline;
  int timeline_capacity;
  int timeline_written; /* out: entries written by block 0 */
} cesa_report;

#define CESA_TL_STEP 1       /* a pose update starts */
#define CESA_TL_WAIT 2       /* first streamed chunk of a sweep has landed */
#define CESA_TL_COMPUTE 3    /* a unit's affinity loop is done */
#define CESA_TL_UNIT 4       /* a unit's reduction / completion is done */
#define CESA_TL_SYNC 5       /* a grid barrier has been passed */
#define CESA_TL_REDUCE 6     /* block partials reduced */
#define CESA_TL_POSE 7       /* pose solved */

/* Reference defaults: src/main.cpp:280-315 (moutlier = e^-1 / sqrt(T_0)). */
void cesa_params_default(cesa_params* p);

/*
 * Annealed EM-ICP. Replaces emicp(), src/emicp.cu:247-716 (declared at
 * src/3dregistration.h:87-90). X: N target points, Y: M source points, host
 * SoA. R, t: host, in/out. Synchronous; device memory is cached between calls.
 */
int cesa_emicp(const float* X, int N, const float* Y, int M, float R[9], float t[3],
               const cesa_params* p, cesa_report* rep);

/*
 * Annealed Softassign. Replaces softassign(), src/softassign.cu:256-886
 * (declared at src/3dregistration.h:82-86). Same conventions as cesa_emicp.
 */
int cesa_softassign(const float* X, int N, const float* Y, int M, float R[9], float t[3],
                    const cesa_params* p, cesa_report* rep);

/*
 * Device-pointer variants (same algorithms as above, inputs already in HBM).
 * dX, dY: device SoA. dRt: device float[12] = R row-major then t, in/out.
 * Enqueued on `stream`; the call returns once the work is queued. The
 * device-side status (CESA_OK or CESA_ERR_TIMEOUT) is written to the device
 * int *d_status when non-NULL, and is also returned by
 * cesa_stream_status(stream) after the stream has been synchronised.
 */
int cesa_emicp_device(const float* dX, int N, const float* dY, int M, float* dRt,
                      const cesa_params* p, int* d_status, cesa_stream_t stream);
int cesa_softassign_device(const float* dX, int N, const float* dY, int M, float* dRt,
                           const cesa_params* p, int* d_status, cesa_stream_t stream);

/* Algorithms of a batched registration (cesa_pair.algorithm). */
#define CESA_ALGO_EMICP 0
#define CESA_ALGO_SOFTASSIGN 1
#define CESA_MAX_BATCH 1024 /* pairs per batched call */

/* One registration of a batch: emicp() or softassign() of X (target) and Y
 * (source), src/3dregistration.h:82-90. X, Y and Rt are device pointers for
 * cesa_register_batch_device and host pointers for cesa_register_batch. Rt
 * holds R (row-major, 9 floats) then t (3): the initial guess on entry, the
 * estimate on return. params: the pair's registrationParameters fields; the
 * sigma_* and d_02 fields drive EM-ICP, JMAX, I0, I1, alpha, T_0, TFACTOR and
 * moutlier drive Softassign. */
typedef struct cesa_pair {
  int algorithm; /* CESA_ALGO_* */
  int N;         /* points in X */
  int M;         /* points in Y */
  const float* X;
  const float* Y;
  float* Rt;
  cesa_params params;
} cesa_pair;

/*
 * Batched registration: every pair of `pairs` (uneven sizes, EM-ICP and
 * Softassign mixed) in one persistent launch, replacing one emicp() or
 * softassign() call per pair. The pairs advance in lock step through their own
 * schedules; each step of every pair is split into (pair, tile) units that all
 * blocks of the GPU share. Each pair's result equals a single-pair call of the
 * same algorithm up to FP32 rounding of the summation order (the Sinkhorn
 * passes complete in a different place). npairs <= CESA_MAX_BATCH. The device
 * variant enqueues on `stream` and writes the device status to *d_status when
 * non-NULL; the host variant copies the clouds in and the poses out and
 * returns when they are written.
 */
int cesa_register_batch_device(const cesa_pair* pairs, int npairs, int* d_status, cesa_stream_t stream);
int cesa_register_batch(const cesa_pair* pairs, int npairs, cesa_report* report);

/*
 * EM-ICP with no device allocation. No counterpart in the reference: this is
 * for callers that cannot call cudaMalloc, such as a plugin inside a host
 * application that owns no device heap, or a real-time pipeline that forbids
 * allocation after start-up. It computes the same result as
 * cesa_emicp_device, bit for bit (same arguments and conventions), but its
 * scratch is a fixed 16 MiB device array inside libcesa.so, held on every GPU
 * that loads the library until the process exits. N = M = 100,000 points fit
 * on a GB300 (the workspace grows with N + M and with the SM count). Larger
 * problems return CESA_ERR_NOALLOC_LIMIT, and nothing is enqueued. The
 * device-side status goes to *d_status when it is non-NULL; either way
 * cesa_stream_status(stream) reports it, read from the fixed scratch, until
 * another call is enqueued on that stream. The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress), so make that first
 * call before any stream capture. Every call on a device shares the one
 * array, which keeps the last call's contents (each call clears what must
 * start at zero): calls that overlap on the GPU (different streams, or a
 * second call enqueued before the first has finished on another stream) race
 * and corrupt each other's results. Serialise them on one stream or
 * synchronise between them. No cudaMalloc, cudaFree or allocating library
 * routine is called.
 */
int cesa_emicp_device_noalloc(const float* dX, int N, const float* dY, int M, float* dRt,
                              const cesa_params* p, int* d_status, cesa_stream_t stream);

/* Status of the last registration enqueued on `stream` (synchronises it);
 * CESA_ERR_INVALID_ARGUMENT when nothing has been enqueued on it. */
int cesa_stream_status(cesa_stream_t stream);

/*
 * ICP: maxIteration iterations of nearest-neighbour matching of the moved
 * source Y to the target X, then Horn's pose (replaces icp(),
 * src/icp.cpp:122-290, declared at src/3dregistration.h:96-99). The
 * reference's FLANN kd-tree search is approximate; this one is exhaustive
 * (exact nearest neighbour; the first of equal distances in X order). Same
 * argument conventions as cesa_emicp; the device variant optionally writes
 * the last iteration's matches (d_nn: M ints, may be NULL).
 */
int cesa_icp(const float* X, int N, const float* Y, int M, float R[9], float t[3], const cesa_params* p,
             cesa_report* report);
int cesa_icp_device(const float* dX, int N, const float* dY, int M, float* dRt, const cesa_params* p,
                    int* d_nn, int* d_status, cesa_stream_t stream);

/*
 * One EM-ICP sigma step (E-step + weighted moments) from pose (R, t): the
 * fused kernel's per-row results for parity checks. Device pointers:
 *   row_out  [M*5]: per Y point r: C_r (row sum incl. outlier term), lambda_r,
 *            lambda_r * X'_r (3)  (may be NULL)
 * Host outputs: moments[16] = sum(lambda), Xc[3], Yc[3], S[9].
 * Replaces one pass of src/emicp.cu:453-624.
 */
int cesa_emicp_step_device(const float* dX, int N, const float* dY, int M, const float R[9],
                           const float t[3], float sigma_p2, float d_02, float* row_out,
                           double moments[16], cesa_stream_t stream);

/*
 * One Softassign inner iteration at temperature T from pose (R, t) and slack
 * (s: N, u: M, device, in/out). Device outputs (may be NULL): rs[N] last row
 * sums incl. slack, cs[M] last column sums incl. slack, w[N] final row sums.
 * Host outputs: moments[16] = sumM, Xc[3], Yc[3], S[9].
 * Replaces one pass of src/softassign.cu:494-798.
 */
int cesa_softassign_step_device(const float* dX, int N, const float* dY, int M, const float R[9],
                                const float t[3], float T, float alpha, int I1, int sinkhorn_form,
                                float* s, float* u, float* rs, float* cs, float* w,
                                double moments[16], cesa_stream_t stream);

/*
 * Horn's pose from the weighted centres and the 3x3 cross-covariance (h_S
 * layout). Replaces findRTfromS(), src/findRTfromS.cpp:33-97 (declared at
 * src/3dregistration.h:104-107). q_prev (nullable, in/out) plays the role of
 * the reference's static q_pre fallback (src/findRTfromS.cpp:110-145).
 * Host function, FP64 internally like the reference.
 */
int cesa_find_rt_from_s(const float Xc[3], const float Yc[3], const float S[9], float R[9],
                        float t[3], float q_prev[4]);

/*
 * AoS points (x,y,z at p[i*stride + 0..2]) to SoA. Replaces cloud2data(),
 * src/cloud2data.cpp:29-67, for callers without PCL.
 */
int cesa_cloud2data(const float* points, int n, int stride_floats, float* soa_out);

/*
 * Autotuner of the Softassign Sinkhorn form. Times the forms (two pose
 * updates each, after a warm-up) on synthetic clouds of N and M points with
 * the schedule parameters of *p (NULL: defaults) on the current device, and
 * records the fastest for the size bucket (half-octaves of N and M). Later
 * calls with sinkhorn_form = CESA_SINKHORN_AUTO and sizes in that bucket use
 * it. Without a recorded decision AUTO uses the banded form where it fits and
 * its grid covers at least half of the SMs with at most 48 bands, else the
 * matrix-free form. The materialised form is skipped when its N x M matrix
 * would take more than half of the free device memory, the banded form where
 * it does not fit. Outputs (may be NULL): the chosen form, the milliseconds
 * per pose update of the matrix-free arithmetic (the faster of the
 * matrix-free and banded decompositions) and of the materialised form (-1
 * when not run). The materialised form, which also holds the N x M matrix, is
 * chosen only when it is at least 10% faster. No counterpart in the
 * reference, which has one (materialised) form.
 */
int cesa_tune_sinkhorn(int N, int M, const cesa_params* p, int* form_out, float* ms_matrix_free,
                       float* ms_materialised);

/*
 * Adjoint of EM-ICP (no counterpart in the reference). A forward pass that
 * also records a tape (per sigma step: input pose, moments, Horn eigenbasis;
 * per step and Y point: C_r, lambda_r, u_r; the packed clouds; no N x M
 * affinity is stored) and a backward pass that, given dL/dR (9, row-major) and
 * dL/dt (3) of the returned pose, writes dL/dX (SoA 3N), dL/dY (SoA 3M) and
 * dL/dR0, dL/dt0 of the initial pose (12). The backward recomputes the
 * affinities step by step. All pointers are device pointers;
 * cesa_emicp_forward_device returns the same pose as cesa_emicp_device. The
 * gradient of a rows' C_r <= 1e-6 branch (lambda = 1, u = mean X) is that of
 * the branch taken, as in any piecewise function.
 */
size_t cesa_emicp_tape_bytes(int N, int M, const cesa_params* p);
int cesa_emicp_forward_device(const float* dX, int N, const float* dY, int M, float* dRt, const cesa_params* p,
                              void* tape, int* d_status, cesa_stream_t stream);
int cesa_emicp_backward_device(int N, int M, const cesa_params* p, const void* tape, const float* d_gRt,
                               float* d_gX, float* d_gY, float* d_gRt0, int* d_status, cesa_stream_t stream);

/*
 * Adjoint of Softassign (no counterpart in the reference). The forward runs
 * the matrix-free kernel (whatever p->sinkhorn_form says) and records a tape:
 * the packed clouds and, per pose update (src/softassign.cu:494-798), its
 * input pose and slack vectors s (N) and u (M), every Sinkhorn pass's
 * scalings, slack and sums (4 (N + M) floats per row and column pass), the
 * final sweep's row sums (5 N) and the Horn solve. The tape is O(N + M) per
 * pass; no N x M matrix is stored. The backward walks the updates in reverse
 * and runs the adjoint of the Horn pose, of the weighted centres and S, and of
 * the column and row passes, forming the affinities on the fly in each K or
 * K^T product and in the two gradient sweeps. One update's launches are
 * replayed as a CUDA graph. Given dL/dR (9, row-major) and dL/dt (3) of the
 * returned pose it writes dL/dX (SoA 3N), dL/dY (SoA 3M) and dL/dR0, dL/dt0 of
 * the initial pose (12). All pointers are device pointers.
 * cesa_softassign_forward_device returns the same pose as
 * cesa_softassign_device with the matrix-free form.
 */
size_t cesa_softassign_tape_bytes(int N, int M, const cesa_params* p);
int cesa_softassign_forward_device(const float* dX, int N, const float* dY, int M, float* dRt,
                                   const cesa_params* p, void* tape, int* d_status, cesa_stream_t stream);
int cesa_softassign_backward_device(int N, int M, const cesa_params* p, const void* tape, const float* d_gRt,
                                    float* d_gX, float* d_gY, float* d_gRt0, int* d_status,
                                    cesa_stream_t stream);

/*
 * Point-cloud front end of the registration CLI (host only; restates the
 * reference CLI's loadFile, pointsReduction, alignScaleOnce, saveRTtoFile and
 * loadRTfromFile, src/main.cpp:41-228, without PCL). Points are AoS xyz.
 *   cesa_load_points: PLY (ASCII / binary, vertex x, y, z of any scalar type)
 *     or text ("x y z" per line); points with a non-finite coordinate are
 *     dropped (as pcl::removeNaNFromPointCloud). *xyz is malloc'ed: release it
 *     with cesa_free.
 *   cesa_points_reduction: keeps each point with probability percent/100, in
 *     order; the reference seeds rand() with the clock, this takes a seed.
 *   cesa_align_scale_once: scales both clouds about the origin so that the
 *     trace of each one's covariance (normalised by n) becomes 0.003.
 *   cesa_save_rt / cesa_load_rt: the reference's R, t text file ("%f " per
 *     entry, three per line, then t).
 * cesa_load_points also reads PCD (PCL's format: DATA ascii, binary or
 * binary_compressed), which the reference's loader reads through PCL.
 *
 * Writers and the rigid transform of the reference's point-cloud tools
 * (src/add_rigid_transform.cpp, src/merge.cpp, src/pcd2ply.cpp):
 *   cesa_save_points: format CESA_POINTS_PCD writes ASCII PCD as PCL's
 *     savePCDFileASCII does (v0.7 header, FIELDS x y z, 8 significant
 *     digits); CESA_POINTS_PLY ASCII PLY (vertex x, y, z float, 8 digits);
 *     CESA_POINTS_TEXT "x y z" lines with 9 digits (exact for FP32);
 *     CESA_POINTS_BY_NAME picks by the extension (.pcd, .ply, else text).
 *   cesa_transform_points: p <- R p + t in place, R row-major; each product
 *     and sum rounded in FP32, left to right, as pcl::transformPointCloud
 *     with an Affine3f.
 */
#define CESA_POINTS_BY_NAME 0
#define CESA_POINTS_PCD 1
#define CESA_POINTS_PLY 2
#define CESA_POINTS_TEXT 3
int cesa_load_points(const char* path, float** xyz, int* n);
void cesa_free(void* p);
int cesa_points_reduction(float* xyz, int* n, float percent, unsigned long long seed);
int cesa_align_scale_once(float* xyz1, int n1, float* xyz2, int n2);
int cesa_save_rt(const char* path, const float R[9], const float t[3]);
int cesa_load_rt(const char* path, float R[9], float t[3]);
int cesa_save_points(const char* path, const float* xyz, int n, int format);
int cesa_transform_points(float* xyz, int n, const float R[9], const float t[3]);

/* Releases cached device workspaces of the calling process. */
void cesa_release_workspaces(void);

/* Human-readable name of a status code. */
const char* cesa_status_string(int status);

/* Self-test of the bounded device-side waits (no counterpart in the
 * reference). Runs, on the current device, the grid barrier (which = 0) or the
 * mbarrier wait (which = 1) used by the registration kernels on a barrier that
 * nothing completes, with a limit of timeout_us microseconds. The wait gives
 * up, records CESA_ERR_TIMEOUT in its control block and returns; *status_out
 * receives that code and *where_out the waiting site's tag. Returns CESA_OK
 * when the probe ran and the device is still usable afterwards. */
int cesa_self_test_waits(int which, int timeout_us, int* status_out, int* where_out);

/* Host-side check of the ranged sweeps' task partition (no counterpart in the
 * reference; needs no GPU): nblk owned blocks of nch tasks each over `grid`
 * blocks, split within SM pairs at pair_num / 256 (0: equal shares; else grid
 * even). Checks, with the functions the kernels use, that the blocks' task
 * ranges tile the tasks in order, that every task maps back to its block,
 * and that every block's slot index among the blocks covering its first owned
 * block is below the partition's kmax (it is the first to cover every later
 * one). Returns CESA_OK, CESA_ERR_INTERNAL when a property fails, or
 * CESA_ERR_INVALID_ARGUMENT; *kmax_out receives kmax. */
int cesa_self_test_partition(int nblk, int nch, int grid, int pair_num, int* kmax_out);

/* Library version as major*10000 + minor*100 + patch. */
int cesa_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CESA_H_ */
