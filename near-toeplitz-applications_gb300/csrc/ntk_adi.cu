// ntk_adi.cu -- Peaceman-Rachford ADI time step (experiments/run-adi.py:59-71).
//
// The reference runs six kernels per step: vertical stencil, row solve,
// transpose, vertical stencil, row solve, transpose (adi/rhs.py:10-25,
// neato.py:8-124, adi/transpose.py:9-27).  Here a step is two fused half
// steps and no transpose:
//   x half: systems = rows 1..N-2 of d_x; RHS = the vertical stencil of u
//           (rows j-1, j, j+1), boundary RHS = d_x's own boundary columns;
//           result written to d_x (as the reference's solve does).
//   y half: systems = columns 1..N-2 of d_x, solved with strided addressing;
//           RHS = the stencil of d_x along its rows (the reference's
//           vertical stencil of u = d_x^T), boundary RHS = d_y's boundary
//           columns; result written straight into u's column, which is
//           where the reference's final transpose puts it.
// In FP64 each half step solves overlapping windows of 32 M rows, one warp
// per window (ntk_adi_f64.cu), when N >= 128 and the factors decay fast
// enough for a halo exact to rounding (r = 0.5: |l| -> 0.268, 36 rows);
// otherwise the segmented FP64 sweeps (ntk_solve_f64.cu) with the largest
// exact segmentation.
// In FP32 + refinement the half steps solve overlapping windows as well
// (ntk_adi_refine.cu); where their factors decay too slowly for an exact
// halo (large r), a step runs the reference's six kernels instead, with the
// partitioned FP32 solve of ntk_spike.cu (nothing truncated) for the rows:
// stencil into d_x, solve, transpose into u, stencil into a work array
// carrying d_y's boundary, solve, transpose into u.
// A whole run of steps can be captured once in a CUDA graph and replayed.
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "ntk_adi_f64.h"
#include "ntk_adi_refine.h"
#include "ntk_internal.h"
#include "ntk_plan.h"
#include "ntk_spike.h"

namespace ntk {

struct Adi {
  int N = 0;
  double dx = 0, dt = 0;
  int precision = NTK_FP64;
  Plan plan;
  double* scratch = nullptr;  // N x N forward values of the segmented sweeps
  SegParams sp;
  double bottom = 0, center = 0, top = 0;
  AdiRefine* refine = nullptr;  // NTK_FP32 / NTK_FP32_REFINE half steps (ntk_adi_refine.cu)
  AdiF64* windows = nullptr;    // NTK_FP64 window half steps (ntk_adi_f64.cu), else segmented sweeps
  SpikeSolver* spike = nullptr;  // FP32 / FP32 + refinement rows where the windows do not apply
  cudaStream_t capture_stream = nullptr;
  std::map<std::tuple<const void*, const void*, const void*, int>, cudaGraphExec_t> graphs;

  ~Adi() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    if (capture_stream) cudaStreamDestroy(capture_stream);
    if (scratch) cudaFree(scratch);
    if (refine) adi_refine_destroy(refine);
    if (windows) adi_f64_destroy(windows);
    if (spike) spike_destroy(spike);
  }
};

namespace {

// Smallest halo H such that every forward window [gL-H, gL) and backward
// window [(g+1)L, (g+1)L+H) has a factor product below 2^-64.
}  // namespace

namespace {

// The boundary of the y half step's work array w, which the final
// transpose turns into u's boundary: rows 0 and N-1 of w are u's columns 0
// and N-1 as they are before the step (so they are not rewritten), columns
// 0 and N-1 of w's rows 1..N-2 are d_y's (the y systems' identity rows).
__global__ void adi_boundary_kernel(const double* __restrict__ u, const double* __restrict__ d_y,
                                    double* __restrict__ w, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const long long row = (long long)i * N;
  w[i] = u[row];
  w[(long long)(N - 1) * N + i] = u[row + N - 1];
  if (i > 0 && i < N - 1) {
    w[row] = d_y[row];
    w[row + N - 1] = d_y[row + N - 1];
  }
}

// experiments/run-adi.py:59-71 with the partitioned FP32 + refinement
// solve: rows 1 .. N-2 of d_x, then of the work array
int adi_spike_step(Adi* a, double* u, double* d_x, const double* d_y, cudaStream_t st) {
  const int N = a->N;
  Batch rows;
  rows.nsys = N - 2;
  rows.ni = N - 2;
  rows.is = N;
  rows.os = 0;
  rows.es = 1;
  adi_boundary_kernel<<<(N + 255) / 256, 256, 0, st>>>(u, d_y, a->scratch, N);
  int rc = cuda_status(cudaGetLastError(), "adi_boundary_kernel");
  if (!rc) rc = launch_adi_rhs(u, d_x, N, a->bottom, a->center, a->top, st);
  if (!rc) rc = spike_solve(a->spike, d_x + N, d_x + N, rows, st);
  if (!rc) rc = launch_transpose2d(d_x, u, N, st);
  if (!rc) rc = launch_adi_rhs(u, a->scratch, N, a->bottom, a->center, a->top, st);
  if (!rc) rc = spike_solve(a->spike, a->scratch + N, a->scratch + N, rows, st);
  if (!rc) rc = launch_transpose2d(a->scratch, u, N, st);
  return rc;
}

}  // namespace

int adi_step(Adi* a, double* u, double* d_x, const double* d_y, cudaStream_t st) {
  if (a->spike) return adi_spike_step(a, u, d_x, d_y, st);
  if (a->refine) return adi_refine_step(a->refine, u, d_x, d_y, st);
  if (a->windows) return adi_f64_step(a->windows, u, d_x, d_y, st);
  const int N = a->N;
  TablesF64 t;
  t.l = a->plan.d_lw;
  t.w = a->plan.d_lw + N;
  int rc = a->plan.g_table(1.0, &t.g);
  if (rc) return rc;
  // x half step
  Batch bx;
  bx.nsys = N - 2;
  bx.ni = N - 2;
  bx.is = N;
  bx.os = 0;
  bx.es = 1;
  RhsParams rx;
  rx.kind = RHS_CROSS;
  rx.bottom = a->bottom;
  rx.center = a->center;
  rx.top = a->top;
  rx.cs = N;
  rx.bnd = d_x + N;
  rx.bnd_ss = N;
  rx.bnd_es = 1;
  rc = launch_thomas_f64_segmented(u + N, a->scratch + N, d_x + N, N, bx, rx, t, a->sp, st);
  if (rc) return rc;
  // y half step
  Batch by;
  by.nsys = N - 2;
  by.ni = N - 2;
  by.is = 1;
  by.os = 0;
  by.es = N;
  RhsParams ry = rx;
  ry.cs = 1;
  ry.bnd = d_y + N;
  ry.bnd_ss = N;
  ry.bnd_es = 1;
  return launch_thomas_f64_segmented(d_x + 1, a->scratch + 1, u + 1, N, by, ry, t, a->sp, st);
}

}  // namespace ntk

struct ntk_adi : public ntk::Adi {};

extern "C" {

int ntk_adi_create(ntk_adi** out, int N, double dx, double dt, int precision) {
  if (!out) {
    ntk::set_error("ntk_adi_create: null out");
    return NTK_ERR_INVALID;
  }
  *out = nullptr;
  if (N < 4 || !(dx > 0) || !(dt > 0) || !std::isfinite(dx) || !std::isfinite(dt)) {
    ntk::set_error("ntk_adi_create: need N >= 4 and positive finite dx, dt");
    return NTK_ERR_INVALID;
  }
  if (precision != NTK_FP64 && precision != NTK_FP32 && precision != NTK_FP32_REFINE) {
    ntk::set_error("ntk_adi_create: unknown precision %d", precision);
    return NTK_ERR_INVALID;
  }
  ntk_adi* a = new (std::nothrow) ntk_adi();
  if (!a) {
    ntk::set_error("ntk_adi_create: out of host memory");
    return NTK_ERR_ALLOC;
  }
  a->N = N;
  a->dx = dx;
  a->dt = dt;
  a->precision = precision;
  // experiments/run-adi.py:50-53 and adi/rhs.py:46-49
  const double co[7] = {1., 0., 1. / (dx * dx), -2. * (1. / dt + 1. / (dx * dx)), 1. / (dx * dx), 0., 1.};
  a->bottom = -1. / (dx * dx);
  a->top = -1. / (dx * dx);
  a->center = 2 * (-1. / dt + 1. / (dx * dx));
  int rc = a->plan.init(N, N - 2, co, NTK_FP64, 1);
  if (rc == NTK_OK) {
    std::vector<double> w(N);
    for (int i = 0; i < N; ++i) w[i] = (i < N - 1 ? a->plan.mat.c(i) : 0.0) / a->plan.lu_u[i];
    a->sp = ntk::choose_segments(a->plan.lu_l.data(), w.data(), N, N - 2);
    if (precision == NTK_FP64) {
      // windows where they apply (N >= 128, fast enough decay), else the
      // segmented sweeps with their N x N scratch array
      rc = ntk::adi_f64_create(&a->windows, N, dx, dt);
      if (rc == NTK_ERR_UNSUPPORTED)
        rc = ntk::cuda_status(cudaMalloc(&a->scratch, sizeof(double) * (size_t)N * N), "cudaMalloc(ADI scratch)");
    } else {
      rc = ntk::adi_refine_create(&a->refine, N, dx, dt, precision);
      if (rc == NTK_ERR_UNSUPPORTED && N > 512) {
        // windows would truncate: exact partitions, the reference's kernel
        // sequence, and two sweeps for the badly conditioned matrices that
        // decay this slowly
        rc = ntk::spike_create(&a->spike, a->plan.mat, precision == NTK_FP32 ? 0 : 2);
        if (!rc)
          rc = ntk::cuda_status(cudaMalloc(&a->scratch, sizeof(double) * (size_t)N * N), "cudaMalloc(ADI work)");
      }
    }
  }
  if (rc) {
    delete a;
    return rc;
  }
  *out = a;
  return NTK_OK;
}

int ntk_adi_destroy(ntk_adi* adi) {
  delete adi;
  return NTK_OK;
}

int ntk_adi_status(ntk_adi* adi, int* flags, void* stream) {
  if (!adi) {
    ntk::set_error("ntk_adi_status: null plan");
    return NTK_ERR_INVALID;
  }
  std::vector<unsigned*> words;
  ntk::adi_refine_status_words(adi->refine, words);
  ntk::spike_status_words(adi->spike, words);
  return ntk::read_clear_status(words, (cudaStream_t)stream, flags);
}

int ntk_adi_segments(const ntk_adi* adi, int* seg_len, int* halo, int* nseg) {
  if (!adi) {
    ntk::set_error("ntk_adi_segments: null plan");
    return NTK_ERR_INVALID;
  }
  if (adi->spike) {
    // partitions of 512 rows, no halo
    if (seg_len) *seg_len = 512;
    if (halo) *halo = 0;
    if (nseg) *nseg = ntk::spike_partitions(adi->spike);
    return NTK_OK;
  }
  if (adi->refine || adi->windows) {
    // windows: central rows per window, halo, windows per system
    int L = 0, H = 0, P = 0;
    if (adi->refine)
      ntk::adi_refine_windows(adi->refine, &L, &H, &P);
    else
      ntk::adi_f64_windows(adi->windows, &L, &H, &P);
    if (seg_len) *seg_len = L;
    if (halo) *halo = H;
    if (nseg) *nseg = P;
    return NTK_OK;
  }
  if (seg_len) *seg_len = adi->sp.L;
  if (halo) *halo = adi->sp.H;
  if (nseg) *nseg = adi->sp.P;
  return NTK_OK;
}

int ntk_adi_step(ntk_adi* adi, double* u, double* d_x, const double* d_y, void* stream) {
  if (!adi || !u || !d_x || !d_y) {
    ntk::set_error("ntk_adi_step: null argument");
    return NTK_ERR_INVALID;
  }
  int rc = adi->plan.check_device();
  if (rc) return rc;
  return ntk::adi_step(adi, u, d_x, d_y, (cudaStream_t)stream);
}

int ntk_adi_run(ntk_adi* adi, double* u, double* d_x, const double* d_y, int steps, int use_graph, void* stream) {
  if (!adi || !u || !d_x || !d_y || steps < 0) {
    ntk::set_error("ntk_adi_run: bad argument");
    return NTK_ERR_INVALID;
  }
  int rc = adi->plan.check_device();
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (!use_graph) {
    for (int s = 0; s < steps; ++s)
      if ((rc = ntk::adi_step(adi, u, d_x, d_y, st))) return rc;
    return NTK_OK;
  }
  auto key = std::make_tuple((const void*)u, (const void*)d_x, (const void*)d_y, steps);
  auto it = adi->graphs.find(key);
  if (it == adi->graphs.end()) {
    // make sure the g table exists before capture (it is uploaded synchronously)
    const double* g = nullptr;
    if ((rc = adi->plan.g_table(1.0, &g))) return rc;
    if (!adi->capture_stream) {
      rc = ntk::cuda_status(cudaStreamCreateWithFlags(&adi->capture_stream, cudaStreamNonBlocking),
                            "cudaStreamCreate(capture)");
      if (rc) return rc;
    }
    rc = ntk::cuda_status(cudaStreamBeginCapture(adi->capture_stream, cudaStreamCaptureModeThreadLocal),
                          "cudaStreamBeginCapture");
    if (rc) return rc;
    int lrc = NTK_OK;
    for (int s = 0; s < steps && lrc == NTK_OK; ++s) lrc = ntk::adi_step(adi, u, d_x, d_y, adi->capture_stream);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(adi->capture_stream, &graph);
    if (lrc) {
      if (graph) cudaGraphDestroy(graph);
      return lrc;
    }
    if ((rc = ntk::cuda_status(e, "cudaStreamEndCapture"))) return rc;
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if ((rc = ntk::cuda_status(e, "cudaGraphInstantiate"))) return rc;
    it = adi->graphs.emplace(key, exec).first;
  }
  return ntk::cuda_status(cudaGraphLaunch(it->second, st), "cudaGraphLaunch");
}

}  // extern "C"
