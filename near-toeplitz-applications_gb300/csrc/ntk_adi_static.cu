// ntk_adi_static.cu -- an ADI time step that allocates nothing.
//
// ntk_adi_create/ntk_adi_step allocate device memory (factor tables and an
// N x N work array for the segmented sweeps) when the plan is built.  Some
// callers cannot do that: code that runs against a fixed, pre-sized memory
// budget that must not grow, hosts with no device allocator, and libraries
// that are handed only the user's buffers and are not allowed to call
// cudaMalloc/cudaFree behind the caller's back.  For them,
// ntk_adi_step_static performs the same step as ntk_adi_step but keeps its
// work array and factor tables in one file-scope __device__ array of fixed
// size, NTK_ADI_STATIC_MAX_N^2 + 3 * NTK_ADI_STATIC_MAX_N doubles (about
// 2 MiB), which every GPU that loads the library holds until the process
// exits.
//
// The array is shared by every call: calls that overlap on the GPU (for
// example on two streams, or from two host threads) race on it.  It keeps the
// last call's contents; every call rewrites the factor tables on its stream
// and every entry of the work array that a call reads is written earlier in
// the same call, so nothing needs clearing.
//
// The factor tables are computed on the host (O(N), no allocation) and handed
// to a one-block kernel by value, in its parameter block (3 N doubles, at
// most 12 KB), which copies them into the array: the values travel with the
// launch, so no host buffer is read after the call returns and no host-device
// copy call is made.
//
// In host code the array's name is only a host-side stand-in, not a device
// address, so the device address is looked up with cudaGetSymbolAddress, once
// per device, by the first call made with that device current, and kept for
// the life of the process (a device reset, cudaDeviceReset included, would
// leave it stale: do not reset a device between calls).  That first call
// should come before any stream capture on the device.
#include <cmath>
#include <mutex>

#include "ntk_internal.h"

namespace ntk {
namespace {

constexpr int kMaxN = NTK_ADI_STATIC_MAX_N;
constexpr int kMaxDevices = 64;

// [0, N*N): work array of the segmented sweeps; then l[N], w[N], g[N]
__device__ __align__(256) double g_adi_static_scratch[(size_t)kMaxN * kMaxN + 3 * kMaxN];

double* g_scratch_addr[kMaxDevices] = {nullptr};

// The factor tables l[N], w[N], g[N] (packed at stride N), passed by value.
struct StaticTables {
  double v[3 * kMaxN];
};

__global__ void adi_static_tables_kernel(const __grid_constant__ StaticTables t, double* dst, int count) {
  for (int i = threadIdx.x; i < count; i += blockDim.x) dst[i] = t.v[i];
}
std::mutex g_scratch_mu;

int scratch_address(int dev, double** out) {
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    int rc = cuda_status(cudaGetSymbolAddress(&p, g_adi_static_scratch), "cudaGetSymbolAddress(ADI scratch)");
    if (rc) return rc;
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return NTK_OK;
}

}  // namespace
}  // namespace ntk

extern "C" int ntk_adi_step_static(int N, double dx, double dt, double* u, double* d_x, const double* d_y,
                                   void* stream) {
  using namespace ntk;
  if (!u || !d_x || !d_y) {
    set_error("ntk_adi_step_static: null array");
    return NTK_ERR_INVALID;
  }
  if (N < 4 || N > kMaxN) {
    set_error("ntk_adi_step_static: N = %d outside 4..%d (the static work array holds N <= %d)", N, kMaxN, kMaxN);
    return NTK_ERR_INVALID;
  }
  if (!(dx > 0) || !(dt > 0) || !std::isfinite(dx) || !std::isfinite(dt)) {
    set_error("ntk_adi_step_static: need positive finite dx, dt");
    return NTK_ERR_INVALID;
  }
  int dev = -1;
  int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("ntk_adi_step_static: device ordinal %d not supported", dev);
    return NTK_ERR_UNSUPPORTED;
  }
  double* scratch = nullptr;
  if ((rc = scratch_address(dev, &scratch))) return rc;

  // Factor tables of experiments/run-adi.py:50-53's matrix, built on the host
  // in the kernel-parameter struct (on the stack, no allocation): l, w, g
  // with g = 1/u.
  StaticTables tabs;
  double* l = tabs.v;
  double* w = tabs.v + N;
  double* g = tabs.v + 2 * N;
  const double a_in = 1. / (dx * dx), b_in = -2. * (1. / dt + 1. / (dx * dx)), c_in = 1. / (dx * dx);
  // rows: 0 = (1, 0), interior = (a_in, b_in, c_in), N-1 = (0, 1)
  double u_prev = 1.0;
  l[0] = 0.0;
  for (int i = 0; i < N; ++i) {
    const double ai = (i == 0 || i == N - 1) ? 0.0 : a_in;
    const double bi = (i == 0 || i == N - 1) ? 1.0 : b_in;
    const double ci_prev = (i - 1 == 0) ? 0.0 : c_in;  // c of row i-1 (row 0 has c = 0)
    double ui = bi;
    if (i > 0) {
      l[i] = ai / u_prev;
      ui = bi - l[i] * ci_prev;
    }
    if (!(ui != 0.0) || !std::isfinite(ui)) {
      set_error("ntk_adi_step_static: zero or non-finite pivot");
      return NTK_ERR_INVALID;
    }
    const double ci = (i == 0 || i == N - 1) ? 0.0 : c_in;
    w[i] = ci / ui;
    g[i] = 1.0 / ui;
    u_prev = ui;
  }
  const SegParams sp = choose_segments(l, w, N, N - 2);

  cudaStream_t st = (cudaStream_t)stream;
  double* dtab = scratch + (size_t)kMaxN * kMaxN;
  adi_static_tables_kernel<<<1, 256, 0, st>>>(tabs, dtab, 3 * N);
  rc = cuda_status(cudaGetLastError(), "adi_static_tables_kernel");
  if (rc) return rc;
  TablesF64 t;
  t.l = dtab;
  t.w = dtab + N;
  t.g = dtab + 2 * N;
  const double bottom = -1. / (dx * dx), top = -1. / (dx * dx), center = 2 * (-1. / dt + 1. / (dx * dx));
  // x half step (rows 1..N-2 of d_x), then y half step (columns 1..N-2, into u)
  Batch bx;
  bx.nsys = N - 2;
  bx.ni = N - 2;
  bx.is = N;
  bx.os = 0;
  bx.es = 1;
  RhsParams rx;
  rx.kind = RHS_CROSS;
  rx.bottom = bottom;
  rx.center = center;
  rx.top = top;
  rx.cs = N;
  rx.bnd = d_x + N;
  rx.bnd_ss = N;
  rx.bnd_es = 1;
  rc = launch_thomas_f64_segmented(u + N, scratch + N, d_x + N, N, bx, rx, t, sp, st);
  if (rc) return rc;
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
  return launch_thomas_f64_segmented(d_x + 1, scratch + 1, u + 1, N, by, ry, t, sp, st);
}
