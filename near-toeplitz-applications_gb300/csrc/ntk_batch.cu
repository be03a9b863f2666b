// ntk_batch.cu -- uneven batches: many independent near-Toeplitz systems of
// different lengths and coefficients, solved in one persistent launch.
//
// Generalises NearToeplitzSolver (neato.py:129-197), which serves one matrix
// of one power-of-two length <= 2048, to a descriptor table: per system a
// length n_s >= 3, an offset into the data buffer, interior coefficients
// (a, b, c) and two special rows at each end.
//
// Factors.  Each system's LU pivots are computed on the host in FP64.  For a
// near-Toeplitz matrix the pivot recurrence u_i = b - (a / u_{i-1}) c reaches
// an exact floating-point fixed point after a few tens of rows; from there on
// every interior row has bit-identical factors, so a system's factor table
// holds only its head rows (up to the fixed point) and its two tail rows, plus
// the converged (l, g, w).  The kernel therefore computes exactly what a
// sequential FP64 Thomas solve with host-computed factors would.
//
// Work distribution.  Systems are sorted by length (longest first) and a
// persistent grid of warps takes them from an atomic counter.  A warp splits
// its system into up to 32 segments, one per lane, when the factors decay
// fast enough for a halo of H rows to be exact to rounding (every halo
// window's factor product below 2^-64): the forward sweep of a segment
// starts H rows early from zero and writes eta to a scratch array; after a
// __syncwarp the backward sweep starts H rows late from zero, reads eta and
// writes x in place.  Systems without enough decay run on one lane.  The
// counter is reset on the stream before every launch, so the launch is
// graph-capturable.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "ntk_batch_refine.h"
#include "ntk_internal.h"
#include "ntk_plan.h"

namespace ntk {

struct SysDesc {
  long long off;  // element offset of row 0 in the data buffer
  int n;          // rows
  int K;          // head rows with tabulated factors (rows K .. n-3 use the converged ones)
  int P;          // segments (lanes)
  int L;          // segment length
  int H;          // halo
  int tab;        // offset of the head table (3K values) followed by the tail rows (6 values)
  double l_inf, g_inf, w_inf;
};

namespace {

__device__ __forceinline__ void row_factors(const SysDesc& sd, const double* __restrict__ pool, int i, double& l,
                                            double& g, double& w) {
  if (i < sd.K) {
    const double* p = pool + sd.tab + 3 * i;
    l = __ldg(p);
    g = __ldg(p + 1);
    w = __ldg(p + 2);
  } else if (i >= sd.n - 2) {
    const double* p = pool + sd.tab + 3 * sd.K + 3 * (i - (sd.n - 2));
    l = __ldg(p);
    g = __ldg(p + 1);
    w = __ldg(p + 2);
  } else {
    l = sd.l_inf;
    g = sd.g_inf;
    w = sd.w_inf;
  }
}

__global__ void __launch_bounds__(128) batch_f64_kernel(double* __restrict__ d, double* __restrict__ scratch,
                                                        const SysDesc* __restrict__ desc,
                                                        const int* __restrict__ order, long long nsys,
                                                        const double* __restrict__ pool, unsigned* counter) {
  const unsigned lane = threadIdx.x & 31;
  for (;;) {
    unsigned item = 0;
    if (lane == 0) item = atomicAdd(counter, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if ((long long)item >= nsys) break;
    const SysDesc sd = desc[order[item]];
    double* x = d + sd.off;
    double* e = scratch + sd.off;
    const int g = (int)lane;
    if (g < sd.P) {
      const int start = g * sd.L;
      const int end = min(sd.n, start + sd.L);
      const int r0 = (g == 0) ? 0 : max(0, start - sd.H);
      double eta = 0.0;
      for (int i = r0; i < end; ++i) {
        double l, gg, w;
        row_factors(sd, pool, i, l, gg, w);
        eta = fma(-l, eta, x[i]);
        if (i >= start) e[i] = eta;
      }
    }
    __syncwarp();
    if (g < sd.P) {
      const int start = g * sd.L;
      const int end = min(sd.n, start + sd.L);
      const int r1 = (g == sd.P - 1) ? sd.n - 1 : min(sd.n - 1, end - 1 + sd.H);
      double xv = 0.0;
      for (int i = r1; i >= start; --i) {
        double l, gg, w;
        row_factors(sd, pool, i, l, gg, w);
        xv = fma(-w, xv, gg * e[i]);
        if (i < end) x[i] = xv;
      }
    }
    __syncwarp();
  }
}

}  // namespace

struct Batch_ {
  long long nsys = 0;
  long long total = 0;  // elements spanned by the data buffer
  int precision = NTK_FP64;
  int device = -1;
  SysDesc* d_desc = nullptr;
  int* d_order = nullptr;
  double* d_pool = nullptr;
  double* d_scratch = nullptr;
  unsigned* d_counter = nullptr;
  int grid = 0;
  long long max_n = 0;
  long long segmented = 0;
  BatchRefine* refine = nullptr;  // NTK_FP32 / NTK_FP32_REFINE windows (ntk_batch_refine.cu)

  ~Batch_() {
    if (refine) batch_refine_destroy(refine);
    if (d_desc) cudaFree(d_desc);
    if (d_order) cudaFree(d_order);
    if (d_pool) cudaFree(d_pool);
    if (d_scratch) cudaFree(d_scratch);
    if (d_counter) cudaFree(d_counter);
  }
};

namespace {

// Host factors of one system; returns false on a zero pivot.
bool system_factors(int n, const double* in3, const double* h6, const double* t6, SysDesc& sd,
                    std::vector<double>& pool) {
  Matrix m;
  m.n = n;
  m.nh = std::min(2, n);
  m.nt = std::min(2, n - m.nh);
  m.ai = in3[0];
  m.bi = in3[1];
  m.ci = in3[2];
  for (int r = 0; r < 2; ++r) {
    m.ha[r] = h6[3 * r];
    m.hb[r] = h6[3 * r + 1];
    m.hc[r] = h6[3 * r + 2];
    m.ta[r] = t6[3 * r];
    m.tb[r] = t6[3 * r + 1];
    m.tc[r] = t6[3 * r + 2];
  }
  if (m.nt < 2) {  // n == 3: one tail row, the last of the given pair
    m.ta[0] = t6[3];
    m.tb[0] = t6[4];
    m.tc[0] = t6[5];
  }
  // sequential LU, stopping at the exact fixed point of the interior
  std::vector<double> l(n, 0.0), u(n, 0.0);
  u[0] = m.b(0);
  if (!(u[0] != 0.0) || !std::isfinite(u[0])) return false;
  int K = n;
  for (int i = 1; i < n; ++i) {
    l[i] = m.a(i) / u[i - 1];
    u[i] = m.b(i) - l[i] * m.c(i - 1);
    if (!(u[i] != 0.0) || !std::isfinite(u[i])) return false;
    if (K == n && i >= 3 && i < n - 2 && u[i] == u[i - 1]) K = i;  // rows >= K share factors
  }
  if (K > n - 2) K = n - 2;
  auto gw = [&](int i, double& g, double& w) {
    g = 1.0 / u[i];
    w = (i < n - 1 ? m.c(i) : 0.0) / u[i];
  };
  sd.n = n;
  sd.K = std::max(0, K);
  sd.tab = (int)pool.size();
  for (int i = 0; i < sd.K; ++i) {
    double g, w;
    gw(i, g, w);
    pool.push_back(l[i]);
    pool.push_back(g);
    pool.push_back(w);
  }
  for (int i = n - 2; i < n; ++i) {
    double g, w;
    gw(i, g, w);
    pool.push_back(l[i]);
    pool.push_back(g);
    pool.push_back(w);
  }
  if (sd.K < n - 2) {
    double g, w;
    gw(sd.K, g, w);
    sd.l_inf = l[sd.K];
    sd.g_inf = g;
    sd.w_inf = w;
  } else {
    sd.l_inf = sd.g_inf = sd.w_inf = 0.0;
  }
  // segmentation: each lane gets >= 4H rows, halo windows must decay below 2^-64
  sd.P = 1;
  sd.L = n;
  sd.H = 0;
  const double lim = std::ldexp(1.0, -64);
  auto fl = [&](int i) { return std::fabs(l[i]); };
  auto fw = [&](int i) { return std::fabs((i < n - 1 ? m.c(i) : 0.0) / u[i]); };
  for (int H = 16; H <= 64 && sd.P == 1; H += 8) {
    int P = std::min(32, n / (4 * H));
    if (P < 2) break;
    const int L = (n + P - 1) / P;
    bool ok = true;
    for (int g = 1; g < P && ok; ++g) {
      double prod = 1.0;
      for (int i = std::max(1, g * L - H); i < g * L; ++i) prod *= fl(i);
      ok = prod <= lim;
    }
    for (int g = 0; g < P - 1 && ok; ++g) {
      double prod = 1.0;
      const int e = std::min(n, (g + 1) * L);
      for (int i = e - 1; i < std::min(n, e + H); ++i) prod *= fw(i);
      ok = prod <= lim;
    }
    if (ok) {
      sd.P = P;
      sd.L = L;
      sd.H = H;
    }
  }
  return true;
}

}  // namespace

}  // namespace ntk

struct ntk_batch : public ntk::Batch_ {};

extern "C" {

int ntk_batch_create(ntk_batch** out, long long nsys, const int* n, const long long* offset, const double* interior,
                     const double* head, const double* tail, int precision) {
  if (!out || nsys < 0 || (nsys > 0 && (!n || !offset || !interior || !head || !tail))) {
    ntk::set_error("ntk_batch_create: null or negative argument");
    return NTK_ERR_INVALID;
  }
  *out = nullptr;
  if (precision != NTK_FP64 && precision != NTK_FP32 && precision != NTK_FP32_REFINE) {
    ntk::set_error("ntk_batch_create: unknown precision %d", precision);
    return NTK_ERR_INVALID;
  }
  if (nsys > 0x7fffffffLL) {
    ntk::set_error("ntk_batch_create: too many systems");
    return NTK_ERR_INVALID;
  }
  ntk_batch* b = new (std::nothrow) ntk_batch();
  if (!b) {
    ntk::set_error("ntk_batch_create: out of host memory");
    return NTK_ERR_ALLOC;
  }
  b->nsys = nsys;
  b->precision = precision;
  std::vector<ntk::SysDesc> desc(nsys);
  std::vector<double> pool;
  long long total = 0;
  for (long long s = 0; s < nsys; ++s) {
    if (n[s] < 3 || offset[s] < 0) {
      ntk::set_error("ntk_batch_create: system %lld has n=%d (need >= 3) or a negative offset", s, n[s]);
      delete b;
      return NTK_ERR_INVALID;
    }
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(interior[3 * s + k])) {
        ntk::set_error("ntk_batch_create: system %lld has a non-finite coefficient", s);
        delete b;
        return NTK_ERR_INVALID;
      }
    desc[s].off = offset[s];
    if (!ntk::system_factors(n[s], interior + 3 * s, head + 6 * s, tail + 6 * s, desc[s], pool)) {
      ntk::set_error("ntk_batch_create: system %lld has a zero or non-finite pivot", s);
      delete b;
      return NTK_ERR_INVALID;
    }
    total = std::max(total, offset[s] + (long long)n[s]);
    b->max_n = std::max(b->max_n, (long long)n[s]);
    b->segmented += desc[s].P > 1;
  }
  // overlapping systems would race
  {
    std::vector<long long> idx(nsys);
    std::iota(idx.begin(), idx.end(), 0LL);
    std::sort(idx.begin(), idx.end(), [&](long long a, long long c) { return offset[a] < offset[c]; });
    for (long long i = 1; i < nsys; ++i)
      if (offset[idx[i - 1]] + n[idx[i - 1]] > offset[idx[i]]) {
        ntk::set_error("ntk_batch_create: systems %lld and %lld overlap", idx[i - 1], idx[i]);
        delete b;
        return NTK_ERR_INVALID;
      }
  }
  std::vector<int> order(nsys);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
    // longest work first (segmented systems split their work over lanes)
    return (double)n[a] / desc[a].P > (double)n[c] / desc[c].P;
  });
  b->total = total;
  int rc = NTK_OK;
  if (cudaGetDevice(&b->device) != cudaSuccess) rc = ntk::cuda_status(cudaGetLastError(), "cudaGetDevice");
  if (pool.empty()) pool.push_back(0.0);
  if (!rc && nsys > 0) {
    rc = ntk::cuda_status(cudaMalloc(&b->d_desc, sizeof(ntk::SysDesc) * nsys), "cudaMalloc(desc)");
    if (!rc) rc = ntk::cuda_status(cudaMalloc(&b->d_order, sizeof(int) * nsys), "cudaMalloc(order)");
    if (!rc) rc = ntk::cuda_status(cudaMalloc(&b->d_pool, sizeof(double) * pool.size()), "cudaMalloc(pool)");
    if (!rc) rc = ntk::cuda_status(cudaMalloc(&b->d_scratch, sizeof(double) * total), "cudaMalloc(scratch)");
    if (!rc) rc = ntk::cuda_status(cudaMalloc(&b->d_counter, sizeof(unsigned)), "cudaMalloc(counter)");
    if (!rc)
      rc = ntk::cuda_status(cudaMemcpy(b->d_desc, desc.data(), sizeof(ntk::SysDesc) * nsys, cudaMemcpyHostToDevice),
                            "cudaMemcpy(desc)");
    if (!rc)
      rc = ntk::cuda_status(cudaMemcpy(b->d_order, order.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice),
                            "cudaMemcpy(order)");
    if (!rc)
      rc = ntk::cuda_status(cudaMemcpy(b->d_pool, pool.data(), sizeof(double) * pool.size(), cudaMemcpyHostToDevice),
                            "cudaMemcpy(pool)");
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    b->grid = sms * 8;  // 8 CTAs of 4 warps per SM, persistent
    if (!rc && precision != NTK_FP64)
      rc = ntk::batch_refine_create(&b->refine, nsys, n, offset, interior, head, tail, precision);
  }
  if (rc) {
    delete b;
    return rc;
  }
  *out = b;
  return NTK_OK;
}

int ntk_batch_destroy(ntk_batch* b) {
  delete b;
  return NTK_OK;
}

int ntk_batch_info(const ntk_batch* b, long long* max_n, long long* segmented, long long* elements) {
  if (!b) {
    ntk::set_error("ntk_batch_info: null batch");
    return NTK_ERR_INVALID;
  }
  if (max_n) *max_n = b->max_n;
  if (segmented) *segmented = b->segmented;
  if (elements) *elements = b->total;
  return NTK_OK;
}

int ntk_batch_solve(ntk_batch* b, double* d, void* stream) {
  if (!b || !d || (reinterpret_cast<uintptr_t>(d) & 7)) {
    ntk::set_error("ntk_batch_solve: null batch or null/misaligned d");
    return NTK_ERR_INVALID;
  }
  if (b->nsys == 0) return NTK_OK;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != b->device) {
    ntk::set_error("ntk_batch_solve: batch was created on device %d, current device is %d", b->device, dev);
    return NTK_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (b->refine) return ntk::batch_refine_solve(b->refine, d, b->d_scratch, b->total, st);
  int rc = ntk::cuda_status(cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), st), "cudaMemsetAsync(counter)");
  if (rc) return rc;
  ntk::batch_f64_kernel<<<b->grid, 128, 0, st>>>(d, b->d_scratch, b->d_desc, b->d_order, b->nsys, b->d_pool,
                                                  b->d_counter);
  return ntk::cuda_status(cudaGetLastError(), "batch_f64_kernel");
}

}  // extern "C"
