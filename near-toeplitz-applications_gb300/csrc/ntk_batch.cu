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
// FP64 windows (batch_f64w_kernel, the default where every system admits
// them): one warp per 512-row window, see the kernel.
//
// Work distribution of the one-warp-per-system kernel (batch_f64_kernel,
// systems whose factors decay too slowly for windows).  Systems are sorted by length (longest first) and a
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

#include "ntk_batch_borders.h"
#include "ntk_batch_refine.h"
#include "ntk_device.cuh"
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

// One FP64 window (batch_f64w_kernel): system rows [w0, w0 + 512), rows
// [lo, hi) of it written back; factors (l, g = 1/u, w = c/u) from the pool:
// Kh head rows at `head`, the system's rows n-2, n-1 at `tail`, (cl, cg, cw)
// elsewhere.
struct F64Win {
  long long off;
  int n, w0, lo, hi;
  int head, Kh, tail, pad_;
  double cl, cg, cw;
  // central rows r < blo or r >= bhi are border rows (a neighbouring window
  // reads them): written to work during the solve, copied into d at the end
  int blo, bhi;
  int sysi, wfirst, wcount;  // the system's counter and windows
  int ccount;                // the system's windows in this window's CTA when it is the first there, else 0
  int rfirst, rcount;        // the system's border rows in the row list (ntk_batch_borders.h)
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

// ---- FP64 windows: one warp per 512-row window of one system ----
// The windows of the FP32 + refinement batch with an FP64 halo (multiplier
// products below 2^-64): systems of up to 512 rows are one window padded
// with identity rows; longer ones overlapping windows whose central rows are
// written back.  Lane j holds window rows [16j, 16j+16) in registers, runs
// Thomas's recurrences over its chunk from zero and applies the chunks'
// carries after an exact affine scan over the lanes (as the FP64 ADI
// windows).  A window's factors differ from the converged interior ones
// only in its first Kh rows (the system's head table for the first window,
// the pivot sequence from a cut for the others, host-tabulated to the exact
// fixed point), the system's last two rows, padding rows and a cut end (c
// dropped); the carry responses are the running products of -l and -c/u.
constexpr int F64W_M = 16;
constexpr int F64W_LW = 32 * F64W_M;
constexpr int F64W_PITCH = 32 * (F64W_M + 1) + 1;  // per-warp tile, chunk pitch M + 1
constexpr int F64W_WARPS = 4;

__device__ __forceinline__ void f64w_fac(const F64Win& w, const double* __restrict__ pool, int r, double& l,
                                         double& g, double& c) {
  const int i = w.w0 + r;
  if (i >= w.n) {  // padding: identity rows
    l = 0.0, g = 1.0, c = 0.0;
    return;
  }
  if (r < w.Kh) {
    const double* p = pool + w.head + 3 * r;
    l = __ldg(p), g = __ldg(p + 1), c = __ldg(p + 2);
  } else if (i >= w.n - 2) {
    const double* p = pool + w.tail + 3 * (i - (w.n - 2));
    l = __ldg(p), g = __ldg(p + 1), c = __ldg(p + 2);
  } else {
    l = w.cl, g = w.cg, c = w.cw;
  }
  if (r == F64W_LW - 1 && i < w.n - 1) c = 0.0;  // cut end
}

// Window wi by one warp, in two parts around a CTA barrier: its rows staged
// from d (coalesced; padding rows zero-filled), then solved and its central
// rows written to d except the border rows, which go to work.
__device__ __forceinline__ void f64_stage(const double* d, const F64Win* __restrict__ wins, long long wi,
                                         double* tile, int lane) {
  constexpr int M = F64W_M;
  const long long base = __ldg(&wins[wi].off) + __ldg(&wins[wi].w0);
  const int rows = __ldg(&wins[wi].n) - __ldg(&wins[wi].w0);
#pragma unroll
  for (int q = 0; q < M; ++q) {
    const int r = lane + 32 * q;
    const bool ok = r < rows;
    cp_async8(tile + (r / M) * (M + 1) + (r % M), ok ? d + base + r : d, ok ? 8u : 0u);
  }
}

__device__ __forceinline__ void f64_window(double* work, double* d, const F64Win* __restrict__ wins,
                                        long long wi, const double* __restrict__ pool, double* tile, int lane) {
  constexpr int M = F64W_M;
  constexpr unsigned FULL = 0xffffffffu;
  const F64Win w = wins[wi];
  const int r0 = lane * M;
  double v[M];
#pragma unroll
  for (int k = 0; k < M; ++k) v[k] = tile[lane * (M + 1) + k];
  double l, g, c;
  // ---- forward ----
  f64w_fac(w, pool, r0, l, g, c);
  double b = -l;
#pragma unroll
  for (int k = 1; k < M; ++k) {
    f64w_fac(w, pool, r0 + k, l, g, c);
    v[k] = fma(-l, v[k - 1], v[k]);
    b *= -l;
  }
  {
    double a = v[M - 1];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double ap = __shfl_up_sync(FULL, a, o);
      const double bp = __shfl_up_sync(FULL, b, o);
      if (lane >= o) {
        a = fma(b, ap, a);
        b *= bp;
      }
    }
    double carry = __shfl_up_sync(FULL, a, 1);
    if (lane == 0) carry = 0.0;
    f64w_fac(w, pool, r0, l, g, c);
    double phi = -l;
    v[0] = fma(phi, carry, v[0]);
#pragma unroll
    for (int k = 1; k < M; ++k) {
      f64w_fac(w, pool, r0 + k, l, g, c);
      phi *= -l;
      v[k] = fma(phi, carry, v[k]);
    }
  }
  // ---- backward ----
  f64w_fac(w, pool, r0 + M - 1, l, g, c);
  v[M - 1] *= g;
  b = -c;
#pragma unroll
  for (int k = M - 2; k >= 0; --k) {
    f64w_fac(w, pool, r0 + k, l, g, c);
    v[k] = fma(-c, v[k + 1], v[k] * g);
    b *= -c;
  }
  {
    double a = v[0];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double ap = __shfl_down_sync(FULL, a, o);
      const double bp = __shfl_down_sync(FULL, b, o);
      if (lane + o < 32) {
        a = fma(b, ap, a);
        b *= bp;
      }
    }
    double carry = __shfl_down_sync(FULL, a, 1);
    if (lane == 31) carry = 0.0;
    f64w_fac(w, pool, r0 + M - 1, l, g, c);
    double psi = -c;
    v[M - 1] = fma(psi, carry, v[M - 1]);
#pragma unroll
    for (int k = M - 2; k >= 0; --k) {
      f64w_fac(w, pool, r0 + k, l, g, c);
      psi *= -c;
      v[k] = fma(psi, carry, v[k]);
    }
  }
  // ---- central rows back through the tile (coalesced) ----
  __syncwarp();
#pragma unroll
  for (int k = 0; k < M; ++k) tile[lane * (M + 1) + k] = v[k];
  __syncwarp();
  const long long base = w.off + w.w0;
  const int blo = __ldg(&wins[wi].blo), bhi = __ldg(&wins[wi].bhi);  // loaded late: not live across the solve
#pragma unroll
  for (int q = 0; q < M; ++q) {
    const int r = lane + 32 * q;
    if (r >= w.lo && r < w.hi) (r < blo || r >= bhi ? work : d)[base + r] = tile[(r / M) * (M + 1) + (r % M)];
  }
}

// All windows in one launch, in place, without a copy of the whole buffer
// and without waiting: a CTA's four windows stage their rows, a CTA barrier,
// then each solves and writes its central rows to d except its border rows
// (central rows a window in another CTA reads, ntk_batch_borders.h), which
// go to work, so d keeps every row another CTA reads unchanged while the
// system's windows run.  After a second barrier the first window of a
// system in the CTA adds the CTA's windows of it to the system's counter;
// the CTA that completes the count copies the system's border rows from work
// into d with all its threads and resets the counter.  Each warp first
// prefetches into L2 the window of the warp pf CTAs further on (pf = the
// CTAs resident at once), so that window's staging finds it in L2.
__global__ void __launch_bounds__(128, 5) batch_f64w_kernel(double* work, double* d, const F64Win* __restrict__ wins,
                                                            long long nwin, const double* __restrict__ pool,
                                                            const long long* __restrict__ border_rows,
                                                            unsigned* done, unsigned pf) {
  __shared__ __align__(16) double tiles[F64W_WARPS * F64W_PITCH];
  __shared__ int last_win[F64W_WARPS];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const long long wi = (long long)blockIdx.x * F64W_WARPS + warp;
  const long long wp = wi + (long long)pf * F64W_WARPS;
  if (lane == 0 && pf > 0 && wp < nwin) {
    const long long base = __ldg(&wins[wp].off) + __ldg(&wins[wp].w0);
    const int rows = min(F64W_LW, __ldg(&wins[wp].n) - __ldg(&wins[wp].w0));
    const uintptr_t a = reinterpret_cast<uintptr_t>(d + base) & ~(uintptr_t)15;
    const uintptr_t e = (reinterpret_cast<uintptr_t>(d + base + rows) + 15) & ~(uintptr_t)15;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((unsigned)(e - a)) : "memory");
  }
  const bool live = wi < nwin;  // every thread reaches the barriers
  double* tile = tiles + warp * F64W_PITCH;
  if (live) f64_stage(d, wins, wi, tile, lane);
  cp_async_wait_all();
  __syncthreads();  // every window of the CTA has read its rows from d
  if (live) f64_window(work, d, wins, wi, pool, tile, lane);
  __syncthreads();  // every window of the CTA has stored its rows
  bool last = false;
  if (live) {
    const int cc = __ldg(&wins[wi].ccount), wcount = __ldg(&wins[wi].wcount);
    if (cc > 0 && cc < wcount) {  // the first window here of a system that other CTAs share
      unsigned l = 0;
      if (lane == 0) {
        __threadfence();
        l = atomicAdd(done + __ldg(&wins[wi].sysi), (unsigned)cc) == (unsigned)(wcount - cc);
        if (l) __threadfence();
      }
      last = __shfl_sync(0xffffffffu, l, 0) != 0;
    }
  }
  if (lane == 0) last_win[warp] = last ? (int)wi : -1;
  __syncthreads();
  for (int k = 0; k < F64W_WARPS; ++k) {
    const int lw = last_win[k];
    if (lw < 0) continue;
    row_copy(work, d, border_rows + __ldg(&wins[lw].rfirst), __ldg(&wins[lw].rcount), (int)threadIdx.x,
             32 * F64W_WARPS);
    if (threadIdx.x == 0) done[__ldg(&wins[lw].sysi)] = 0u;
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
  F64Win* d_wins = nullptr;       // NTK_FP64 windows (batch_f64w_kernel); null: batch_f64_kernel
  long long nwin = 0;

  unsigned* d_done = nullptr;      // per system: its windows finished in the current launch
  long long* d_rows = nullptr;     // the FP64 windows' border rows, grouped by system
  unsigned wpf = 0;                // the window kernel's prefetch distance (CTAs resident at once)

  ~Batch_() {
    if (refine) batch_refine_destroy(refine);
    if (d_wins) cudaFree(d_wins);
    if (d_done) cudaFree(d_done);
    if (d_rows) cudaFree(d_rows);
    if (d_desc) cudaFree(d_desc);
    if (d_order) cudaFree(d_order);
    if (d_pool) cudaFree(d_pool);
    if (d_scratch) cudaFree(d_scratch);
    if (d_counter) cudaFree(d_counter);
  }
};

namespace {

// The matrix of one system: two head rows, the interior, two tail rows (for
// n = 3 the one tail row is the second given one).
void system_matrix(int n, const double* in3, const double* h6, const double* t6, Matrix& m) {
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
}

// Host factors of one system; returns false on a zero pivot.
bool system_factors(int n, const double* in3, const double* h6, const double* t6, SysDesc& sd,
                    std::vector<double>& pool) {
  Matrix m;
  system_matrix(n, in3, h6, t6, m);
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

// Pivot sequence of the window matrix that starts at system row w0 (a
// dropped there): rows (l, g, w) appended to the pool until the exact
// floating-point fixed point inside the interior; K rows, then (cl, cg, cw).
// Returns false on a zero pivot or no fixed point within `limit` rows.
bool cut_sequence(const Matrix& m, int w0, int limit, std::vector<double>& pool, int& K, double conv[3]) {
  const int n = m.n;
  double u = m.b(w0);
  if (!(u != 0.0) || !std::isfinite(u)) return false;
  pool.push_back(0.0);
  pool.push_back(1.0 / u);
  pool.push_back((w0 < n - 1 ? m.c(w0) : 0.0) / u);
  for (int i = w0 + 1; i < n && i - w0 <= limit; ++i) {
    const double l = m.a(i) / u;
    const double un = m.b(i) - l * m.c(i - 1);
    if (!(un != 0.0) || !std::isfinite(un)) return false;
    const double w = (i < n - 1 ? m.c(i) : 0.0) / un;
    if (i >= w0 + 3 && i < n - 2 && un == u) {
      K = i - w0;
      conv[0] = l, conv[1] = 1.0 / un, conv[2] = w;
      return true;
    }
    pool.push_back(l);
    pool.push_back(1.0 / un);
    pool.push_back(w);
    u = un;
  }
  return false;
}

// FP64 windows of one system (see batch_f64w_kernel), appended to `wins`;
// false when the factors decay too slowly for 128 central rows per window.
bool system_windows(int n, const double* in3, const double* h6, const double* t6, const SysDesc& sd, int sysi,
                    std::vector<double>& pool, std::vector<F64Win>& wins, int& count) {
  constexpr int LW = F64W_LW;
  F64Win base{};
  base.off = sd.off;
  base.n = n;
  base.tail = sd.tab + 3 * sd.K;
  count = 0;
  if (n <= LW) {  // one window, padded with identity rows
    F64Win w = base;
    w.w0 = 0, w.lo = 0, w.hi = n;
    w.blo = 0, w.bhi = n;  // a whole system: no border rows
    w.sysi = sysi, w.wfirst = (int)wins.size(), w.wcount = 1;
    w.head = sd.tab, w.Kh = sd.K;
    w.cl = sd.l_inf, w.cg = sd.g_inf, w.cw = sd.w_inf;
    wins.push_back(w);
    count = 1;
    return true;
  }
  if (sd.K > LW / 4) return false;
  Matrix m;
  system_matrix(n, in3, h6, t6, m);
  // interior cuts share one sequence (started at row 2, the first interior row)
  int Kc = 0;
  double cc[3];
  const int cut_tab = (int)pool.size();
  if (!cut_sequence(m, 2, LW / 4, pool, Kc, cc)) return false;
  // halo: multiplier products below 2^-64 from a cut start (forward) and
  // before a cut end (backward, |w| converged), plus two
  const double lim = std::ldexp(1.0, -64);
  int hf = 0, hb = 0;
  for (double p = 1.0; p > lim && hf < 4 * LW; ++hf)
    p *= std::fabs(hf + 1 < Kc ? pool[cut_tab + 3 * (hf + 1)] : cc[0]);
  for (double p = 1.0; p > lim && hb < 4 * LW; ++hb) p *= std::fabs(cc[2]);
  const int H = (std::max(hf, hb) + 2 + 1) & ~1;
  const int L = LW - 2 * H;
  if (L < LW / 4) return false;
  auto add = [&](int w0, int lo, int hi, int head, int Kh, const double* cv) {
    F64Win w = base;
    w.w0 = w0, w.lo = lo, w.hi = hi, w.head = head, w.Kh = Kh;
    w.cl = cv[0], w.cg = cv[1], w.cw = cv[2];
    wins.push_back(w);
    ++count;
  };
  const double sc[3] = {sd.l_inf, sd.g_inf, sd.w_inf};
  add(0, 0, LW - H, sd.tab, sd.K, sc);
  int pos = LW - H;
  const int last_w0 = n - LW;
  const int last_lo = last_w0 + H;
  while (pos < last_lo) {
    const int w0 = pos - H;
    const int hi = std::min(pos + L, last_lo);
    add(w0, pos - w0, hi - w0, cut_tab, Kc, cc);
    pos = hi;
  }
  if (last_w0 >= 2) {
    add(last_w0, pos - last_w0, LW, cut_tab, Kc, cc);
  } else {  // n = 513: the last window starts at a head row
    int Kl = 0;
    double cl[3];
    const int tab = (int)pool.size();
    if (!cut_sequence(m, last_w0, LW / 4, pool, Kl, cl)) return false;
    add(last_w0, pos - last_w0, LW, tab, Kl, cl);
  }
  // the system's windows; border rows are set for the whole list
  // (ntk_batch_borders.h) once every system has its windows
  const size_t first = wins.size() - count;
  for (int g = 0; g < count; ++g) {
    F64Win& w = wins[first + g];
    w.sysi = sysi;
    w.wfirst = (int)first;
    w.wcount = count;
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
  // FP64: windows, one warp each, when every system admits them (else the
  // persistent one-warp-per-system kernel)
  std::vector<ntk::F64Win> wins;
  std::vector<long long> border_rows;
  if (precision == NTK_FP64) {
    long long multi = 0;
    bool ok = true;
    for (long long s = 0; s < nsys && ok; ++s) {
      int count = 0;
      ok = ntk::system_windows(n[s], interior + 3 * s, head + 6 * s, tail + 6 * s, desc[s], (int)s, pool, wins, count);
      multi += count > 1;
    }
    if (ok) {
      b->segmented = multi;
      ntk::cta_borders(
          wins, ntk::F64W_WARPS, ntk::F64W_LW, [](const ntk::F64Win& w) { return w.off + w.w0; },
          [](const ntk::F64Win& w) { return w.lo; }, [](const ntk::F64Win& w) { return w.hi; }, border_rows);
    } else {
      wins.clear();
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
    if (!rc && !wins.empty()) {
      b->nwin = (long long)wins.size();
      rc = ntk::cuda_status(cudaMalloc(&b->d_wins, sizeof(ntk::F64Win) * wins.size()), "cudaMalloc(windows)");
      if (!rc)
        rc = ntk::cuda_status(
            cudaMemcpy(b->d_wins, wins.data(), sizeof(ntk::F64Win) * wins.size(), cudaMemcpyHostToDevice),
            "cudaMemcpy(windows)");
    }
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    b->grid = sms * 8;  // 8 CTAs of 4 warps per SM, persistent
    if (!rc && b->d_wins) {
      int per_sm = 0;
      rc = ntk::cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ntk::batch_f64w_kernel,
                                                                          32 * ntk::F64W_WARPS, 0),
                            "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
      b->wpf = (unsigned)(per_sm * sms);
      if (!rc)
        rc = ntk::cuda_status(cudaMalloc(&b->d_done, sizeof(unsigned) * (size_t)nsys), "cudaMalloc(system counters)");
      if (!rc)
        rc = ntk::cuda_status(cudaMemset(b->d_done, 0, sizeof(unsigned) * (size_t)nsys), "cudaMemset(system counters)");
      if (!rc && !border_rows.empty()) {
        rc = ntk::cuda_status(cudaMalloc(&b->d_rows, sizeof(long long) * border_rows.size()), "cudaMalloc(border rows)");
        if (!rc)
          rc = ntk::cuda_status(cudaMemcpy(b->d_rows, border_rows.data(), sizeof(long long) * border_rows.size(),
                                           cudaMemcpyHostToDevice),
                                "cudaMemcpy(border rows)");
      }
    }
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

int ntk_batch_status(ntk_batch* b, int* flags, void* stream) {
  if (!b) {
    ntk::set_error("ntk_batch_status: null batch");
    return NTK_ERR_INVALID;
  }
  std::vector<unsigned*> words;
  if (b->refine) ntk::batch_refine_status_words(b->refine, words);
  return ntk::read_clear_status(words, (cudaStream_t)stream, flags);
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

int ntk_batch_windows(const ntk_batch* b, long long* windows, long long* paired) {
  if (!b) {
    ntk::set_error("ntk_batch_windows: null batch");
    return NTK_ERR_INVALID;
  }
  long long w = 0, p = 0;
  if (b->refine) {
    w = ntk::batch_refine_windows(b->refine);
    p = ntk::batch_refine_paired_windows(b->refine);
  } else if (b->d_wins) {
    w = b->nwin;
  }
  if (windows) *windows = w;
  if (paired) *paired = p;
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
  if (b->refine) return ntk::batch_refine_solve(b->refine, d, b->d_scratch, st);
  if (b->d_wins) {
    // one launch: windows solved in place, border rows through work
    const long long blocks = (b->nwin + ntk::F64W_WARPS - 1) / ntk::F64W_WARPS;
    ntk::batch_f64w_kernel<<<(unsigned)blocks, 32 * ntk::F64W_WARPS, 0, st>>>(b->d_scratch, d, b->d_wins, b->nwin,
                                                                              b->d_pool, b->d_rows, b->d_done, b->wpf);
    return ntk::cuda_status(cudaGetLastError(), "batch_f64w_kernel");
  }
  int rc = ntk::cuda_status(cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), st), "cudaMemsetAsync(counter)");
  if (rc) return rc;
  ntk::batch_f64_kernel<<<b->grid, 128, 0, st>>>(d, b->d_scratch, b->d_desc, b->d_order, b->nsys, b->d_pool,
                                                  b->d_counter);
  return ntk::cuda_status(cudaGetLastError(), "batch_f64_kernel");
}

}  // extern "C"
