/*
 * ntk.h -- C ABI of libntk, the GB300-native (sm_103a) batched near-Toeplitz
 * tridiagonal solver with the compact finite-difference and ADI operators
 * around it.
 *
 * Drop-in boundary for the hot path of ashwinsrnth/near-toeplitz-applications:
 * plain pointers and sizes, no C++ or torch types.  Device pointers are CUDA
 * device addresses of the calling process's current device; `stream` is a
 * cudaStream_t (NULL = legacy default stream, as the reference uses).  Every
 * call is asynchronous with respect to the host unless stated otherwise and
 * returns an ntk_status; ntk_last_error() returns the message of the last
 * failure on the calling thread.
 *
 * Matrices follow the reference's model (neato.py:131-139): coeffs =
 * (b1, c1, ai, bi, ci, an, bn), row 0 = [b1 c1], rows 1..n-2 = [ai bi ci],
 * row n-1 = [an bn].  n >= 3; unlike the reference, n need not be a power
 * of two and is not capped at 2048.
 */
#ifndef NTK_H
#define NTK_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum ntk_status {
  NTK_OK = 0,
  NTK_ERR_INVALID = 1,     /* bad argument (size, pointer, stride, mode) */
  NTK_ERR_CUDA = 2,        /* a CUDA runtime call or launch failed */
  NTK_ERR_UNSUPPORTED = 3, /* valid request this build does not serve */
  NTK_ERR_RANGE = 4,       /* input magnitude outside the FP32+refine range */
  NTK_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
  NTK_ERR_ALLOC = 6        /* host or device allocation failed */
} ntk_status;

typedef enum ntk_precision {
  NTK_FP64 = 0,            /* plain FP64 solve */
  NTK_FP32 = 1,            /* FP32 solve only (no refinement) */
  NTK_FP32_REFINE = 2      /* FP32 solves + double-word residual refinement */
} ntk_precision;

typedef struct ntk_plan ntk_plan;

/* Version string of the library build. */
const char* ntk_version(void);

/* Message of the last failed call on this thread ("" if none).  Copies at
 * most len-1 bytes plus a terminating NUL into buf; returns the full length. */
int ntk_last_error(char* buf, int len);

/* Builds a solver for systems of length n with the reference's coefficient
 * tuple.  Replaces NearToeplitzSolver.__init__ (neato.py:131-166): the
 * per-level CR coefficient arrays of _precompute_coefficients
 * (neato.py:199-274) become the shared matrix's LU factors, computed once in
 * FP64 on the host and uploaded.  nrhs is the number of contiguous systems
 * ntk_solve works on (neato.py:135-136).  precision is an ntk_precision;
 * refine_sweeps (>= 1) is used by NTK_FP32_REFINE.  FP32 paths: n <= 1024
 * runs one warp per system; longer systems run as overlapping 512-row
 * windows (NTK_ERR_UNSUPPORTED when the LU multipliers |a/u|, |c/u| of the
 * interior are >= 0.9, too slow a decay for the windows), and an in-place
 * call on them copies its input to a work array the plan allocates on first
 * use.  Synchronous. */
int ntk_plan_create(ntk_plan** out, int n, long long nrhs, const double coeffs[7], int precision,
                    int refine_sweeps);

/* Launch configuration of a plan (what the reference fixes in its jinja2
 * templates, neato.py:160-163): set by the autotuner (ntk/autotune.py) or by
 * hand.  Keys and values:
 *   NTK_TUNE_F64_X_VARIANT  contiguous FP64 sweeps: 0 transposing tile ring
 *                           (default), 1 whole-system shared tile, 2 direct
 *   NTK_TUNE_F64_THREADS    threads per block of the one-thread-per-system
 *                           FP64 kernel: 32, 64, 128 (default)
 *   NTK_TUNE_REFINE_W       warps per CTA of the FP32+refine kernel: 4,
 *                           8 (default) or 16 (kernel variants with one
 *                           system per warp, n <= 512 and one sweep; the
 *                           others, and the windowed n > 1024 kernel, run
 *                           8)
 *   NTK_TUNE_REFINE_SPW     systems per warp of that kernel: 1 (default) or
 *                           2 (strided layouts with n in 257..512 only; a
 *                           CTA then stages twice as many adjacent systems)
 *   NTK_TUNE_REFINE_KERNEL  n = 512, one sweep or none: the paired-chunk
 *                           kernels with TMA tiles where the matrix and the
 *                           layout allow them (power-of-two interior,
 *                           16-byte aligned buffers, even strides), with
 *                           strided layouts either one 16-system group per
 *                           CTA (2) or in persistent CTAs, one per SM, two
 *                           groups solved while a third loads (3); 0
 *                           (default) picks 3 for NTK_FP32 and 2 for
 *                           NTK_FP32_REFINE (faster on GB300); 1 the
 *                           chunked kernel above.  With 0, 2 or 3,
 *                           NTK_TUNE_REFINE_W sets the systems per CTA of
 *                           contiguous layouts (4, 8 or 16).
 *   NTK_TUNE_REFINE_PREFETCH  the one-group strided kernel: a CTA prefetches
 *                           into L2 the tile the CTA resident p / 2 waves
 *                           later will load, p = 0 (none) .. 4; default 2
 *                           (one wave).
 *   NTK_TUNE_REFINE_TPS     threads per system for 512 < n <= 1024: 32 (one
 *                           warp, 32 rows per lane; 0 = default) or 64 (two
 *                           overlapping 512-row windows, 16 rows per lane,
 *                           where the factors decay fast enough; else 32). */
enum ntk_tune_key {
  NTK_TUNE_F64_X_VARIANT = 1,
  NTK_TUNE_F64_THREADS = 2,
  NTK_TUNE_REFINE_W = 3,
  NTK_TUNE_REFINE_SPW = 4,
  NTK_TUNE_REFINE_KERNEL = 5,
  NTK_TUNE_REFINE_PREFETCH = 6,
  NTK_TUNE_REFINE_TPS = 7
};
int ntk_plan_set_tuning(ntk_plan* plan, int key, int value);
int ntk_plan_get_tuning(const ntk_plan* plan, int key, int* value);

/* Frees the plan's device tables.  Synchronous; NULL is accepted. */
int ntk_plan_destroy(ntk_plan* plan);

/* Status of the plan's solves since the last status read.  The FP32 and
 * FP32+refine kernels cannot represent |x| >= 2^128 (nor inf or nan) in
 * their double-word arithmetic (and keep only FP32 accuracy for a system
 * whose largest |x| is below about 2^-80, which is not flagged: scale such
 * data by a power of two, which every operation preserves exactly, or use
 * NTK_FP64); when a solve meets an input at or above 2^128 it still
 * completes, with a meaningless result, and raises NTK_STATUS_RANGE in a
 * device status word of the plan.  This call reads that word on `stream`
 * (after every solve issued before it on that stream), clears it, waits for
 * the stream and stores the bits in *flags (flags may be NULL).  Returns
 * NTK_ERR_RANGE when NTK_STATUS_RANGE is set, NTK_OK otherwise; FP64 plans
 * always report 0.  The reference validates only n (neato.py:145); this
 * extends its error reporting to the value range.  Synchronous. */
#define NTK_STATUS_RANGE 1
int ntk_plan_status(ntk_plan* plan, int* flags, void* stream);

/* Solves plan->nrhs contiguous systems in place: d[s*n + k], 0 <= s < nrhs.
 * Replaces NearToeplitzSolver.solve(x_d) (neato.py:168-197); d may be a
 * pointer-offset view into a larger buffer, as in experiments/run-adi.py:65. */
int ntk_solve(ntk_plan* plan, double* d, void* stream);

/* Solves nsys systems laid out with strides (in elements): system s starts at
 * (s / ni) * os + (s % ni) * is and its k-th unknown is es further on per k.
 * The y and z sweeps of a C-ordered [nz][ny][nx] field are
 *   y: ni = nx, is = 1, os = nx*ny, es = nx      (nsys = nz*nx)
 *   z: ni = nx*ny, is = 1, os = 0, es = nx*ny    (nsys = ny*nx)
 * which removes the permutes of experiments/run-compact.py:70-73,83-86.
 * In place (d_out == d_in) or out of place with the same layout. */
int ntk_solve_strided(ntk_plan* plan, const double* d_in, double* d_out, long long nsys, long long ni,
                      long long is, long long os, long long es, void* stream);

/* Compact 4th-order first derivative of an [nz][ny][nx] FP64 field along
 * axis (0 = z, 1 = y, 2 = x), grid spacing h: the RHS of compact/rhs.py:9-37
 * fused into the solve's load phase, with strided addressing for y and z.
 * Replaces compute_rhs + solve (experiments/run-compact.py:57-60) and, for
 * y/z, the two permutes around them (run-compact.py:67-90).  The plan's n
 * must equal the extent of the chosen axis; nrhs is ignored.  out must not
 * overlap f unless out == f. */
int ntk_compact_deriv(ntk_plan* plan, const double* f, double* out, int nz, int ny, int nx, int axis, double h,
                      void* stream);

/* The three compact derivatives of an n x n x n field (nz = ny = nx = the
 * plan's n) into three separate arrays: the whole of
 * experiments/run-compact.py:47-90 in one call.  For n = 512 on the
 * NTK_FP32 / NTK_FP32_REFINE paths of the paired-chunk solve this is ONE
 * kernel launch: per z-plane its x and y groups run side by side (the plane
 * is read from HBM once for both), then the z groups; otherwise it is three
 * ntk_compact_deriv calls.  f and the outputs must not overlap. */
int ntk_compact_grad(ntk_plan* plan, const double* f, double* dfdx, double* dfdy, double* dfdz, int nz, int ny,
                     int nx, double h, void* stream);

/* compute_rhs(f, rhs, dx) of compact/rhs.py:47-53: the RHS along the last
 * axis of an [nz][ny][nx] field.  Any nz, ny >= 1 and nx >= 3 (the
 * reference needs multiples of 8). */
int ntk_compact_rhs(const double* f, double* rhs, int nz, int ny, int nx, double dx, void* stream);

/* permute(a_d, b_d, permutation) of compact/permute.py:32-52:
 * out[i0][i1][i2] = in[i0*s0 + i1*s1 + i2*s2] with out of shape (o0, o1, o2)
 * and (s0, s1, s2) the input's element strides in permutation order. */
int ntk_permute3d(const double* in, double* out, int o0, int o1, int o2, long long s0, long long s1, long long s2,
                  void* stream);

/* compute_rhs(u, d, dx, dt, N) of adi/rhs.py:35-55: interior points of d get
 * bottom*u[i-N] + center*u[i] + top*u[i+N] with the reference's dx, dt
 * coefficients (adi/rhs.py:46-49); boundary points of d are untouched. */
int ntk_adi_rhs(const double* u, double* d, int N, double dx, double dt, void* stream);

/* transpose(a, b, N) of adi/transpose.py:40-50: b = a^T for N x N FP64. */
int ntk_transpose2d(const double* a, double* b, int N, void* stream);

/* ---- ADI (Peaceman-Rachford) heat equation on an N x N grid ------------
 * One step replaces the six launches of experiments/run-adi.py:59-71
 * (compute_rhs, solve, transpose, twice) with two fused half steps and no
 * transpose.  The matrix is the reference's (run-adi.py:50-53):
 * (1, 0, 1/dx^2, -2(1/dt + 1/dx^2), 1/dx^2, 0, 1), RHS stencil adi/rhs.py:46-49. */
typedef struct ntk_adi ntk_adi;

/* Builds the ADI solver for N x N fields (N >= 4).  precision:
 *   NTK_FP64         FP64 over overlapping 32M-row windows, one warp per
 *                    window (halos exact to FP64 rounding), when N >= 128 and
 *                    the factors decay fast enough; otherwise segmented FP64
 *                    sweeps with an N x N FP64 work array.
 *   NTK_FP32_REFINE  FP32 solve + one double-word refinement sweep per half
 *                    step, over overlapping 32M-row windows (M = 16, 8 or 4;
 *                    needs N >= 128, else NTK_ERR_UNSUPPORTED); matches the
 *                    FP64 path to ~1e-13.  Where the factors decay too slowly
 *                    for the windows' halos (large dt / dx^2) and N > 512:
 *                    the reference's six kernels per step with an exact
 *                    partitioned FP32 solve (512-row partitions coupled by a
 *                    reduced system, two sweeps; N <= 8192) and an N x N
 *                    work array.
 *   NTK_FP32         the same without the refinement sweeps.
 * Synchronous. */
int ntk_adi_create(ntk_adi** out, int N, double dx, double dt, int precision);

int ntk_adi_destroy(ntk_adi* adi);

/* ntk_plan_status for the ADI plan's FP32 / FP32+refine half steps (FP64
 * plans report 0).  Synchronous. */
int ntk_adi_status(ntk_adi* adi, int* flags, void* stream);

/* The segmentation the plan chose: for windows (NTK_FP32, NTK_FP32_REFINE,
 * and NTK_FP64 where they apply) the windows' central rows, halo and windows
 * per system; for the partitioned FP32 solve 512, 0 and the partitions per
 * system; for the segmented FP64 sweeps segment length, halo and segments
 * per system (1 segment = plain sweeps). */
int ntk_adi_segments(const ntk_adi* adi, int* seg_len, int* halo, int* nseg);

/* One time step on device arrays u, d_x, d_y (N x N, C order), with the
 * reference's meaning: afterwards u is the reference's u after one loop
 * iteration and rows 1..N-2 of d_x hold the x half step's solution.  d_y is
 * read only at its boundary columns (0 and N-1 of rows 1..N-2); its interior,
 * scratch in the reference, is not written.  u's boundary columns are not
 * rewritten: with the reference's initialisation d_y = u^T
 * (run-adi.py:45-46) they already hold the values the reference's last
 * transpose would put there. */
int ntk_adi_step(ntk_adi* adi, double* u, double* d_x, const double* d_y, void* stream);

/* `steps` time steps.  use_graph != 0 captures the steps once per
 * (u, d_x, d_y, steps) into a CUDA graph and replays it on later calls. */
int ntk_adi_run(ntk_adi* adi, double* u, double* d_x, const double* d_y, int steps, int use_graph, void* stream);

/* ---- ADI with per-line coefficients ----------------------------------------
 * Generalises the reference's single ADI matrix (run-adi.py:50-53, the
 * model of neato.py:136-138) to one near-Toeplitz system per line:
 * u_t = kx(y) u_xx + ky(x) u_yy, kx[j] the x diffusivity on row j, ky[i] the
 * y diffusivity on column i (kx = ky = 1 is the reference's step).  A step
 * follows run-adi.py:59-71: the stencil of adi/rhs.py:21-24 with per-column
 * coefficients (-k/dx^2, 2(-1/dt + k/dx^2), -k/dx^2) into d_x, the rows
 * 1..N-2 of d_x solved with (1, 0 | a, -2(1/dt + a), a | 0, 1), a = k/dx^2 of
 * their own line (uneven batches: FP64 windows, or FP32 + refinement
 * windows with NTK_FP32_REFINE), u = d_x^T, and the same into d_y, u = d_y^T.
 * d_x and d_y keep their boundary values (the reference initialises d_x = u,
 * d_y = u^T).  Create and destroy are synchronous. */
typedef struct ntk_adi_var ntk_adi_var;
int ntk_adi_var_create(ntk_adi_var** out, int N, double dx, double dt, const double* kx, const double* ky,
                       int precision);
int ntk_adi_var_destroy(ntk_adi_var* adi);
int ntk_adi_var_step(ntk_adi_var* adi, double* u, double* d_x, double* d_y, void* stream);
/* ntk_plan_status for the per-line batches' FP32 windows.  Synchronous. */
int ntk_adi_var_status(ntk_adi_var* adi, int* flags, void* stream);

/* ---- ADI step that allocates nothing ----------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory (code running against a fixed, pre-sized memory budget, hosts with
 * no device allocator, libraries that may only touch the buffers they are
 * given): the same
 * step as ntk_adi_step without a plan, with its work array and factor tables
 * in one static device array of NTK_ADI_STATIC_MAX_N^2 + 3 NTK_ADI_STATIC_MAX_N
 * doubles (~2 MiB, held by every GPU that loads the library until exit).
 * N above NTK_ADI_STATIC_MAX_N is rejected with NTK_ERR_INVALID.  Calls no
 * cudaMalloc/cudaFree.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) and keeps it for the life of the process (do
 * not reset the device between calls); make that first call before any
 * stream capture.  All
 * calls share the array: calls that overlap on the GPU race.  The factor
 * tables are computed on the host by every call and written into the array
 * on `stream` by a one-block kernel that receives them by value in its
 * parameter block (no host buffer is read after the call returns). */
#define NTK_ADI_STATIC_MAX_N 512
int ntk_adi_step_static(int N, double dx, double dt, double* u, double* d_x, const double* d_y, void* stream);

/* ---- uneven batches ------------------------------------------------------
 * nsys independent near-Toeplitz systems of different lengths and
 * coefficients in one buffer, solved in place by one launch.
 * Generalises NearToeplitzSolver (neato.py:129-197: one matrix, one
 * power-of-two n <= 2048) to a descriptor table.  System s: n[s] >= 3 rows
 * starting at element offset[s]; interior rows (a, b, c) =
 * interior[3s .. 3s+2]; rows 0 and 1 = head[6s .. 6s+5] as (a, b, c) pairs
 * (a of row 0 ignored); rows n-2 and n-1 = tail[6s .. 6s+5] (c of row n-1
 * ignored).  Systems must not overlap. */
typedef struct ntk_batch ntk_batch;

/* Factors every system on the host (FP64) and uploads the tables; allocates
 * a work array as large as the data buffer.  precision: NTK_FP64 (overlapping
 * 512-row windows, one warp each, exact to FP64 rounding, when every system's
 * factors converge and decay fast enough; otherwise one warp per system), or
 * NTK_FP32_REFINE / NTK_FP32: systems cut into overlapping 512-row windows
 * solved in FP32 with one double-word refinement sweep (NTK_ERR_UNSUPPORTED
 * when some system's pivots decay too slowly, |a/u|, |c/u| >= 0.75).
 * Synchronous. */
int ntk_batch_create(ntk_batch** out, long long nsys, const int* n, const long long* offset, const double* interior,
                     const double* head, const double* tail, int precision);

int ntk_batch_destroy(ntk_batch* batch);

/* ntk_plan_status for an uneven batch's FP32 / FP32+refine windows (FP64
 * batches report 0).  Synchronous. */
int ntk_batch_status(ntk_batch* batch, int* flags, void* stream);

/* Longest system, number of systems split over several windows (or, on the
 * one-warp-per-system FP64 path, over several lanes), and the number of
 * elements the data buffer must span. */
int ntk_batch_info(const ntk_batch* batch, long long* max_n, long long* segmented, long long* elements);

/* Windows the batch solves (512 rows each, one warp per window; 0 on the
 * one-warp-per-system FP64 path) and, for NTK_FP32_REFINE / NTK_FP32, how
 * many of them take the paired-chunk FP32 solve (constant Toeplitz factors
 * with end corrections; the others, and systems shorter than 512 rows, take
 * the chunked solve with per-window factor tables). */
int ntk_batch_windows(const ntk_batch* batch, long long* windows, long long* paired);

/* Solves every system in place in d (device), asynchronously on `stream`:
 * windows (FP64 windows, NTK_FP32_REFINE, NTK_FP32) are one kernel launch
 * (each window reads its rows from d and writes its central rows back; the
 * rows a neighbouring window reads go through the work array until the
 * system's last window copies them in); the one-warp-per-system FP64 kernel
 * is one launch preceded by a 4-byte memset of its work counter.
 * Graph-capturable. */
int ntk_batch_solve(ntk_batch* batch, double* d, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NTK_H */
