// ntk_solve_f64.cu -- plain FP64 batched near-Toeplitz solves.
//
// Replaces the reference's sharedMemCyclicReduction (neato.py:8-124) and,
// for the fused variants, its computeRHS (compact/rhs.py:9-37) and
// applyVerticalStencil (adi/rhs.py:10-25) launches, plus the permutes and
// transposes the drivers wrap around them (experiments/run-compact.py:67-90,
// experiments/run-adi.py:59-71).
//
// Design for GB300.  The FP64 pipe of a GB300 SM retires ~1.7 DFMA/DADD per
// clock (1/72 of FP32) with a 64-cycle latency, so this path is bound by
// FP64 instructions, not by HBM.  Every system shares one matrix, so its LU
// factors are computed once on the host (l_i, g_i = s/u_i, w_i = c_i/u_i)
// and each thread runs the Thomas recurrences on one system:
//   forward   eta_i = D_i - l_i * eta_{i-1}          (1 DFMA; +1 DADD for the
//                                                      compact RHS difference)
//   backward  x_i  = g_i * eta_i - w_i * x_{i+1}     (1 DMUL off the chain + 1 DFMA)
// i.e. 3 (in-place solve) or 4 (fused compact derivative) FP64 instructions
// per unknown, against ~10 plus two FP64 divisions per unknown in the
// reference's cyclic reduction.  The forward values eta are parked in the
// output array (they are L2-resident until the backward pass overwrites them
// with x), so no shared memory is needed and occupancy is set by registers.
// Threads of a warp take adjacent systems: for y/z sweeps of a 3D field these
// are adjacent x-columns, so every row access is one coalesced 256-byte
// segment and no permute pass is needed.
#include <cstdio>

#include "ntk_device.cuh"
#include "ntk_internal.h"

namespace ntk {
namespace {

constexpr int PF = 8;  // rows prefetched ahead of the recurrence

// ----------------------------------------------------------------------------
// row streams: forward (ascending) and backward (descending) with a register
// prefetch ring, so load latency overlaps the recurrence.
// ----------------------------------------------------------------------------
template <bool VEC>
struct FwdStream {
  const double* p;
  long long es;
  int n;
  double ring[PF];
  __device__ __forceinline__ void init(const double* src, long long stride, int len) {
    p = src;
    es = stride;
    n = len;
    if constexpr (VEC) {
#pragma unroll
      for (int k = 0; k < PF; k += 2) {
        if (k + 1 < n) {
          double2 v = *reinterpret_cast<const double2*>(p + k);
          ring[k] = v.x;
          ring[k + 1] = v.y;
        } else if (k < n) {
          ring[k] = p[k];
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < PF; ++k)
        if (k < n) ring[k] = p[(long long)k * es];
    }
  }
  // value of row i (ring slot i % PF); refills the slot with row i + PF
  __device__ __forceinline__ double take(const int K, int i) {
    double v = ring[K];
    if constexpr (VEC) {
      if ((K & 1) == 1) {
        // refill the pair (i+PF-1, i+PF) once both slots are consumed
        int j = i - 1 + PF;
        if (j + 1 < n) {
          double2 q = *reinterpret_cast<const double2*>(p + j);
          ring[K - 1] = q.x;
          ring[K] = q.y;
        } else if (j < n) {
          ring[K - 1] = p[j];
        }
      }
    } else {
      if (i + PF < n) ring[K] = p[(long long)(i + PF) * es];
    }
    return v;
  }
};

// ----------------------------------------------------------------------------
// forward sweeps
// ----------------------------------------------------------------------------
// Identity RHS: eta_i = d_i - l_i eta_{i-1}; eta stored into dst.
template <bool VEC>
__device__ __forceinline__ double forward_identity(const double* src, double* dst, long long es, int n,
                                                   const double* __restrict__ l) {
  FwdStream<VEC> st;
  st.init(src, es, n);
  double eta = 0.0;
  int i0 = 0;
  for (; i0 + PF <= n; i0 += PF) {
#pragma unroll
    for (int k = 0; k < PF; ++k) {
      const int i = i0 + k;
      const double v = st.take(k, i);
      eta = (i == 0) ? v : fma(-__ldg(l + i), eta, v);
      dst[(long long)i * es] = eta;
    }
  }
#pragma unroll
  for (int k = 0; k < PF; ++k) {  // tail (< PF rows), no refill needed
    const int i = i0 + k;
    if (i < n) {
      const double v = st.ring[k];
      eta = (i == 0) ? v : fma(-__ldg(l + i), eta, v);
      dst[(long long)i * es] = eta;
    }
  }
  return eta;
}

// Compact 4th-order RHS fused into the forward sweep, in eta units (y / s):
//   eta_0     = sigma0 * ((-5 f0 + 4 f1) + f2)
//   eta_i     = (f_{i+1} - f_{i-1}) - l_i eta_{i-1}                1 <= i <= n-2
//   eta_{n-1} = sigmaN * ((-5 f_{n-1} + 4 f_{n-2}) + f_{n-3}) - l_{n-1} eta_{n-2}
// Row i is finished when f_{i+1} arrives; the f window lives in registers so
// dst may alias src.
template <bool VEC>
__device__ __forceinline__ double forward_compact(const double* src, double* dst, long long es, int n,
                                                  const double* __restrict__ l, double sigma0, double sigmaN) {
  FwdStream<VEC> st;
  st.init(src, es, n);
  double fa = 0.0, fb = 0.0;  // f_{j-2}, f_{j-1}
  double eta = 0.0;
  auto consume = [&](int j, double fc) {
    if (j == 0) {
      fb = fc;
    } else if (j == 1) {
      fa = fb;
      fb = fc;
    } else {
      if (j == 2) {
        eta = sigma0 * ((-5.0 * fa + 4.0 * fb) + fc);
        dst[0] = eta;
      }
      eta = fma(-__ldg(l + (j - 1)), eta, fc - fa);
      dst[(long long)(j - 1) * es] = eta;
      fa = fb;
      fb = fc;
    }
  };
  int i0 = 0;
  for (; i0 + PF <= n; i0 += PF) {
#pragma unroll
    for (int k = 0; k < PF; ++k) {
      const int i = i0 + k;
      const double v = st.take(k, i);
      consume(i, v);
    }
  }
#pragma unroll
  for (int k = 0; k < PF; ++k)
    if (i0 + k < n) consume(i0 + k, st.ring[k]);
  return eta;  // eta_{n-2}; the caller closes row n-1
}

// ----------------------------------------------------------------------------
// backward sweep: x_i = g_i eta_i - w_i x_{i+1}, eta read back from dst.
// ----------------------------------------------------------------------------
template <bool VEC>
__device__ __forceinline__ void backward(double* dst, long long es, int n, double eta_last,
                                         const double* __restrict__ g, const double* __restrict__ w) {
  double x = __ldg(g + (n - 1)) * eta_last;
  dst[(long long)(n - 1) * es] = x;
  // descending prefetch ring over rows n-2 ... 0
  double ring[PF];
#pragma unroll
  for (int k = 0; k < PF; ++k) {
    const int i = n - 2 - k;
    if (i >= 0) ring[k] = dst[(long long)i * es];
  }
  int r0 = 0;  // ring position of row n-2-r0
  for (; r0 + PF <= n - 1; r0 += PF) {
#pragma unroll
    for (int k = 0; k < PF; ++k) {
      const int i = n - 2 - (r0 + k);
      const double e = ring[k];
      const int ip = i - PF;
      if (ip >= 0) ring[k] = dst[(long long)ip * es];
      x = fma(-__ldg(w + i), x, __ldg(g + i) * e);
      dst[(long long)i * es] = x;
    }
  }
#pragma unroll
  for (int k = 0; k < PF; ++k) {
    const int i = n - 2 - (r0 + k);
    if (i >= 0) {
      x = fma(-__ldg(w + i), x, __ldg(g + i) * ring[k]);
      dst[(long long)i * es] = x;
    }
  }
}

template <int RHS, bool VEC>
__global__ void __launch_bounds__(128) thomas_f64_kernel(const double* in, double* out, int n, Batch b,
                                                         RhsParams rp, TablesF64 t) {
  const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.nsys) return;
  const long long base = (s / b.ni) * b.os + (s % b.ni) * b.is;
  const double* src = in + base;
  double* dst = out + base;
  double eta;
  if constexpr (RHS == RHS_IDENTITY) {
    eta = forward_identity<VEC>(src, dst, b.es, n, t.l);
  } else {
    // keep the last three f values for the closing boundary row
    const double fl0 = src[(long long)(n - 3) * b.es];
    const double fl1 = src[(long long)(n - 2) * b.es];
    const double fl2 = src[(long long)(n - 1) * b.es];
    eta = forward_compact<VEC>(src, dst, b.es, n, t.l, rp.sigma0, rp.sigmaN);
    // eta currently holds eta_{n-2}; close with row n-1
    eta = fma(-__ldg(t.l + (n - 1)), eta, rp.sigmaN * ((-5.0 * fl2 + 4.0 * fl1) + fl0));
    dst[(long long)(n - 1) * b.es] = eta;
  }
  backward<VEC>(dst, b.es, n, eta, t.g, t.w);
}

// ----------------------------------------------------------------------------
// segmented sweeps for batches with few, long systems (the ADI half-steps:
// 2046 systems of 2048 rows).  One thread per (segment, system); adjacent
// threads take adjacent systems of the same segment, so strided layouts stay
// coalesced.  Forward: eta over [start - H, end) from zero, stored for
// [start, end) into `eta`; backward: x over (end + H, start] from zero, read
// from `eta`, stored for [start, end) into `out`.  eta and out are distinct
// buffers, so neighbouring segments never race.
// ----------------------------------------------------------------------------
template <int RHS>
__device__ __forceinline__ double seg_rhs(const double* __restrict__ in, long long p, int i, int n, long long s,
                                          const RhsParams& rp) {
  if constexpr (RHS == RHS_CROSS) {
    if (i == 0) return rp.bnd[s * rp.bnd_ss];
    if (i == n - 1) return rp.bnd[s * rp.bnd_ss + (long long)(n - 1) * rp.bnd_es];
    return fma(rp.top, in[p + rp.cs], fma(rp.center, in[p], rp.bottom * in[p - rp.cs]));
  } else {
    return in[p];
  }
}

template <int RHS>
__global__ void __launch_bounds__(128) seg_fwd_kernel(const double* __restrict__ in, double* __restrict__ eta,
                                                      int n, Batch b, RhsParams rp, const double* __restrict__ l,
                                                      SegParams sp) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= b.nsys * sp.P) return;
  const int g = (int)(gt / b.nsys);
  const long long s = gt % b.nsys;
  const long long base = (s / b.ni) * b.os + (s % b.ni) * b.is;
  const int start = g * sp.L;
  const int end = min(n, start + sp.L);
  const int r0 = (g == 0) ? 0 : max(0, start - sp.H);
  double e = 0.0;
#pragma unroll 8
  for (int i = r0; i < end; ++i) {
    const long long p = base + (long long)i * b.es;
    e = fma(-__ldg(l + i), e, seg_rhs<RHS>(in, p, i, n, s, rp));
    if (i >= start) eta[p] = e;
  }
}

__global__ void __launch_bounds__(128) seg_bwd_kernel(const double* __restrict__ eta, double* __restrict__ out,
                                                      int n, Batch b, const double* __restrict__ gt_,
                                                      const double* __restrict__ w, SegParams sp) {
  const long long gt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gt >= b.nsys * sp.P) return;
  const int g = (int)(gt / b.nsys);
  const long long s = gt % b.nsys;
  const long long base = (s / b.ni) * b.os + (s % b.ni) * b.is;
  const int start = g * sp.L;
  const int end = min(n, start + sp.L);
  const int r1 = (g == sp.P - 1) ? n - 1 : min(n - 1, end - 1 + sp.H);
  double x = 0.0;
#pragma unroll 8
  for (int i = r1; i >= start; --i) {
    const long long p = base + (long long)i * b.es;
    x = fma(-__ldg(w + i), x, __ldg(gt_ + i) * eta[p]);
    if (i < end) out[p] = x;
  }
}

// ----------------------------------------------------------------------------
// contiguous (x-direction) systems: stage a tile of 32 systems in shared
// memory with coalesced loads, run the recurrences from shared memory with
// one lane per system (pitch n + 1 doubles: lanes hit distinct banks), and
// store the tile coalesced.  eta and x overwrite the tile in place.
// ----------------------------------------------------------------------------
template <int RHS>
__global__ void __launch_bounds__(32) thomas_f64_staged_kernel(const double* __restrict__ in, double* __restrict__ out,
                                                               int n, Batch b, RhsParams rp, TablesF64 t) {
  extern __shared__ __align__(16) double tile[];
  const int lane = threadIdx.x;
  const int pitch = n + 1;
  const long long s0 = (long long)blockIdx.x * 32;
  const int cnt = (int)min(32LL, b.nsys - s0);
  // stage: one system at a time, lanes walk its rows; cp.async keeps every
  // copy of the tile in flight at once
  for (int w = 0; w < cnt; ++w) {
    const long long s = s0 + w;
    const double* src = in + (s / b.ni) * b.os + (s % b.ni) * b.is;
    double* trow = tile + w * pitch;
#pragma unroll 4
    for (int r = lane; r < n; r += 32) cp_async8(trow + r, src + r, 8u);
  }
  cp_async_wait_all();
  __syncwarp();
  if (lane < cnt) {
    // Rows are processed in blocks of 8: the block's loads are issued
    // together ahead of its dependent FMA chain (the chain, not the loads,
    // bounds the loop).
    constexpr int B = 8;
    double* v = tile + lane * pitch;
    double eta;
    if constexpr (RHS == RHS_IDENTITY) {
      eta = v[0];
      for (int i0 = 1; i0 < n; i0 += B) {
        double fv[B], lv[B];
#pragma unroll
        for (int k = 0; k < B; ++k) {
          const int i = min(i0 + k, n - 1);
          fv[k] = v[i];
          lv[k] = __ldg(t.l + i);
        }
#pragma unroll
        for (int k = 0; k < B; ++k) {
          if (i0 + k < n) {
            eta = fma(-lv[k], eta, fv[k]);
            v[i0 + k] = eta;
          }
        }
      }
    } else {
      const double f0 = v[0], f1 = v[1], f2 = v[2];
      const double fl0 = v[n - 3], fl1 = v[n - 2], fl2 = v[n - 1];
      eta = rp.sigma0 * ((-5.0 * f0 + 4.0 * f1) + f2);
      double fm = f0, fc = f1;  // f_{i-1}, f_i
      v[0] = eta;
      for (int i0 = 1; i0 < n - 1; i0 += B) {
        double fv[B], lv[B];
#pragma unroll
        for (int k = 0; k < B; ++k) {
          const int i = min(i0 + k, n - 2);
          fv[k] = v[i + 1];
          lv[k] = __ldg(t.l + i);
        }
#pragma unroll
        for (int k = 0; k < B; ++k) {
          if (i0 + k < n - 1) {
            eta = fma(-lv[k], eta, fv[k] - fm);
            v[i0 + k] = eta;
            fm = fc;
            fc = fv[k];
          }
        }
      }
      eta = fma(-__ldg(t.l + (n - 1)), eta, rp.sigmaN * ((-5.0 * fl2 + 4.0 * fl1) + fl0));
      v[n - 1] = eta;
    }
    double x = __ldg(t.g + (n - 1)) * eta;
    v[n - 1] = x;
    for (int i0 = n - 2; i0 >= 0; i0 -= B) {
      double ev[B], gv[B], wv[B];
#pragma unroll
      for (int k = 0; k < B; ++k) {
        const int i = max(i0 - k, 0);
        ev[k] = v[i];
        gv[k] = __ldg(t.g + i);
        wv[k] = __ldg(t.w + i);
      }
#pragma unroll
      for (int k = 0; k < B; ++k) {
        if (i0 - k >= 0) {
          x = fma(-wv[k], x, gv[k] * ev[k]);
          v[i0 - k] = x;
        }
      }
    }
  }
  __syncwarp();
  for (int w = 0; w < cnt; ++w) {
    const long long s = s0 + w;
    double* dst = out + (s / b.ni) * b.os + (s % b.ni) * b.is;
    const double* trow = tile + w * pitch;
#pragma unroll 4
    for (int r = lane; r < n; r += 32) dst[r] = trow[r];
  }
}

// ----------------------------------------------------------------------------
// contiguous (x-direction) systems, many at a time: each warp takes 32
// adjacent systems and moves their rows through a per-warp ring of 32 x 33
// shared-memory tiles.  Loads and stores touch one system's 32 consecutive
// rows per instruction (coalesced 256 B), the recurrence reads the tile
// transposed (lane = system; pitch 33 keeps both directions conflict-free).
// cp.async keeps the next tiles in flight while the current one is solved.
// Forward: f tiles in, eta tiles out (parked in `out`); backward: eta tiles
// in, x tiles out.  Needs es == 1 and the 32 systems of a warp to be
// equally spaced (is), which the launcher checks.
// ----------------------------------------------------------------------------
constexpr int XT = 16;       // rows per tile
constexpr int XP = 33;       // tile pitch (doubles): one row of the tile holds 32 systems + 1 pad
constexpr int XRING = 3;     // tiles in flight per warp
constexpr int XWARPS = 4;    // warps per CTA
constexpr int XSUB = 32 / XT;  // systems covered by one warp instruction of the tile copies

// tile[row][w] <- system w, global row row0 + row: lanes cover XT rows of
// XSUB systems per instruction (coalesced XT*8-byte segments)
__device__ __forceinline__ void xtile_issue(double* tile, const double* base0, long long is, int cnt, int row0, int n,
                                            int lane) {
  const int k = lane % XT;
  const int ws = lane / XT;
  const int r = row0 + k;
  const bool ok = r < n;
#pragma unroll 8
  for (int w0 = 0; w0 < 32; w0 += XSUB) {
    const int w = w0 + ws;
    const bool v = ok && (w < cnt);
    cp_async8(tile + k * XP + w, base0 + (v ? (long long)w * is + r : 0), v ? 8u : 0u);
  }
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void xtile_store(const double* tile, double* base0, long long is, int cnt, int row0, int n,
                                            int lane) {
  const int k = lane % XT;
  const int ws = lane / XT;
  const int r = row0 + k;
  if (r < n) {
#pragma unroll 8
    for (int w0 = 0; w0 < 32; w0 += XSUB) {
      const int w = w0 + ws;
      if (w < cnt) base0[(long long)w * is + r] = tile[k * XP + w];
    }
  }
}

template <int RHS>
__global__ void __launch_bounds__(32 * XWARPS) thomas_f64_xpose_kernel(const double* in, double* out, int n, Batch b,
                                                                       RhsParams rp, TablesF64 t) {
  extern __shared__ __align__(16) double xsm[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  double* ring = xsm + (size_t)warp * XRING * XT * XP;
  const long long s0 = ((long long)blockIdx.x * XWARPS + warp) * 32;
  if (s0 >= b.nsys) return;  // whole warp
  const int cnt = (int)min(32LL, b.nsys - s0);
  const long long off0 = (s0 / b.ni) * b.os + (s0 % b.ni) * b.is;
  const double* src = in + off0;
  double* dst = out + off0;
  const int C = (n + XT - 1) / XT;

  // ---- forward: eta_i, tiles of f in, tiles of eta out ----
  double eta = 0.0;
  double fm = 0.0, fc = 0.0;  // compact: f_{i-1}, f_i
  double fl0 = 0.0, fl1 = 0.0, fl2 = 0.0;
  xtile_issue(ring, src, b.is, cnt, 0, n, lane);
  if (C > 1) xtile_issue(ring + XT * XP, src, b.is, cnt, XT, n, lane);
  for (int c = 0; c < C; ++c) {
    double* cur = ring + (c % XRING) * XT * XP;
    const double* nxt = ring + ((c + 1) % XRING) * XT * XP;
    // tiles c and c+1 must be complete (the compact RHS of the tile's last
    // row needs the next tile's first row); only tile c+2 may stay in flight
    if (c + 2 < C) {
      xtile_issue(ring + ((c + 2) % XRING) * XT * XP, src, b.is, cnt, (c + 2) * XT, n, lane);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncwarp();
    const int row0 = c * XT;
    const int rows = min(XT, n - row0);
    if constexpr (RHS == RHS_IDENTITY) {
#pragma unroll 8
      for (int k = 0; k < rows; ++k) {
        const int i = row0 + k;
        const double v = cur[k * XP + lane];
        eta = (i == 0) ? v : fma(-__ldg(t.l + i), eta, v);
        cur[k * XP + lane] = eta;
      }
    } else {
      if (c == 0) {
        fm = cur[0 * XP + lane];
        fc = cur[1 * XP + lane];
        eta = rp.sigma0 * ((-5.0 * fm + 4.0 * fc) + cur[2 * XP + lane]);
      }
#pragma unroll 8
      for (int k = 0; k < rows; ++k) {
        const int i = row0 + k;
        if (i == 0) {
          cur[lane] = eta;
          continue;
        }
        if (i == n - 1) {
          eta = fma(-__ldg(t.l + i), eta, rp.sigmaN * ((-5.0 * fl2 + 4.0 * fl1) + fl0));
          cur[k * XP + lane] = eta;
          continue;
        }
        // f_{i+1}: next row of this tile or the first row of the next tile
        const double fp = (k + 1 < XT) ? cur[(k + 1) * XP + lane] : nxt[lane];
        if (i == n - 3) fl0 = fc;
        eta = fma(-__ldg(t.l + i), eta, fp - fm);
        fm = fc;
        fc = fp;
        if (i == n - 2) {
          fl1 = fm;
          fl2 = fc;
        }
        cur[k * XP + lane] = eta;
      }
    }
    __syncwarp();
    xtile_store(cur, dst, b.is, cnt, row0, n, lane);
    __syncwarp();
  }
  // ---- backward: x_i = g_i eta_i - w_i x_{i+1}, tiles of eta in (from out) ----
  // each lane reads back exactly the rows it stored; the fence orders those
  // stores before the asynchronous copies that read them
  __threadfence_block();
  double x = 0.0;
  xtile_issue(ring, dst, b.is, cnt, (C - 1) * XT, n, lane);
  if (C > 1) xtile_issue(ring + XT * XP, dst, b.is, cnt, (C - 2) * XT, n, lane);
  for (int cc = 0; cc < C; ++cc) {
    const int c = C - 1 - cc;
    double* cur = ring + (cc % XRING) * XT * XP;
    if (cc + 2 < C) {
      xtile_issue(ring + ((cc + 2) % XRING) * XT * XP, dst, b.is, cnt, (c - 2) * XT, n, lane);
      asm volatile("cp.async.wait_group 2;\n" ::: "memory");
    } else if (cc + 1 < C) {
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncwarp();
    const int row0 = c * XT;
    const int rows = min(XT, n - row0);
#pragma unroll 8
    for (int k = rows - 1; k >= 0; --k) {
      const int i = row0 + k;
      const double e = cur[k * XP + lane];
      x = (i == n - 1) ? __ldg(t.g + i) * e : fma(-__ldg(t.w + i), x, __ldg(t.g + i) * e);
      cur[k * XP + lane] = x;
    }
    __syncwarp();
    xtile_store(cur, dst, b.is, cnt, row0, n, lane);
    __syncwarp();
  }

}

}  // namespace

int launch_thomas_f64(const double* in, double* out, int n, const Batch& b, const RhsParams& rp,
                      const TablesF64& t, int threads, cudaStream_t stream, int x_variant) {
  if (b.nsys <= 0) return NTK_OK;
  if (threads <= 0 || threads > 128 || threads % 32) threads = 128;
  const long long blocks = (b.nsys + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) {
    set_error("too many systems for one launch");
    return NTK_ERR_INVALID;
  }
  // double2 loads need unit element stride, 16-byte aligned system starts
  bool vec = (b.es == 1) && (n % 2 == 0) && (b.is % 2 == 0) && (b.os % 2 == 0) &&
             ((reinterpret_cast<uintptr_t>(in) & 15) == 0) && ((reinterpret_cast<uintptr_t>(out) & 15) == 0);
  dim3 grid((unsigned)blocks), block(threads);
  // contiguous systems, 32 per warp equally spaced: transposing tile ring
  const bool xlike = (b.es == 1) && (b.ni >= b.nsys || b.ni % 32 == 0) && (rp.kind == RHS_IDENTITY || n >= 4) &&
                     (rp.kind == RHS_IDENTITY || rp.kind == RHS_COMPACT);
  if (xlike && x_variant == 0) {
    const size_t xs = (size_t)XWARPS * XRING * XT * XP * sizeof(double);
    const long long xblocks = (b.nsys + 32 * XWARPS - 1) / (32 * XWARPS);
    if (rp.kind == RHS_IDENTITY) {
      auto k = thomas_f64_xpose_kernel<RHS_IDENTITY>;
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xs);
      k<<<(unsigned)xblocks, 32 * XWARPS, xs, stream>>>(in, out, n, b, rp, t);
    } else {
      auto k = thomas_f64_xpose_kernel<RHS_COMPACT>;
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xs);
      k<<<(unsigned)xblocks, 32 * XWARPS, xs, stream>>>(in, out, n, b, rp, t);
    }
    return cuda_status(cudaGetLastError(), "thomas_f64_xpose_kernel");
  }
  // contiguous systems that fit a 32-system tile in shared memory: staged kernel
  const size_t smem = (size_t)32 * (n + 1) * sizeof(double);
  if (b.es == 1 && smem <= 200 * 1024 && (rp.kind == RHS_IDENTITY || rp.kind == RHS_COMPACT) &&
      (rp.kind == RHS_IDENTITY || n >= 4) && x_variant != 2) {
    const long long sblocks = (b.nsys + 31) / 32;
    if (rp.kind == RHS_IDENTITY) {
      auto k = thomas_f64_staged_kernel<RHS_IDENTITY>;
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k<<<(unsigned)sblocks, 32, smem, stream>>>(in, out, n, b, rp, t);
    } else {
      auto k = thomas_f64_staged_kernel<RHS_COMPACT>;
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k<<<(unsigned)sblocks, 32, smem, stream>>>(in, out, n, b, rp, t);
    }
    return cuda_status(cudaGetLastError(), "thomas_f64_staged_kernel");
  }
  if (rp.kind == RHS_IDENTITY) {
    if (vec)
      thomas_f64_kernel<RHS_IDENTITY, true><<<grid, block, 0, stream>>>(in, out, n, b, rp, t);
    else
      thomas_f64_kernel<RHS_IDENTITY, false><<<grid, block, 0, stream>>>(in, out, n, b, rp, t);
  } else if (rp.kind == RHS_COMPACT) {
    if (vec)
      thomas_f64_kernel<RHS_COMPACT, true><<<grid, block, 0, stream>>>(in, out, n, b, rp, t);
    else
      thomas_f64_kernel<RHS_COMPACT, false><<<grid, block, 0, stream>>>(in, out, n, b, rp, t);
  } else {
    set_error("unsupported RHS kind %d for the FP64 solve", rp.kind);
    return NTK_ERR_INVALID;
  }
  return cuda_status(cudaGetLastError(), "thomas_f64_kernel");
}

}  // namespace ntk

namespace ntk {

int launch_thomas_f64_segmented(const double* in, double* eta, double* out, int n, const Batch& b,
                                const RhsParams& rp, const TablesF64& t, const SegParams& sp, cudaStream_t stream) {
  if (b.nsys <= 0) return NTK_OK;
  if (sp.P < 1 || sp.L < 1 || (long long)sp.L * sp.P < n || sp.H < 0) {
    set_error("bad segmentation (L=%d H=%d P=%d, n=%d)", sp.L, sp.H, sp.P, n);
    return NTK_ERR_INVALID;
  }
  const int threads = 128;
  const long long blocks = (b.nsys * sp.P + threads - 1) / threads;
  if (rp.kind == RHS_CROSS)
    seg_fwd_kernel<RHS_CROSS><<<(unsigned)blocks, threads, 0, stream>>>(in, eta, n, b, rp, t.l, sp);
  else if (rp.kind == RHS_IDENTITY)
    seg_fwd_kernel<RHS_IDENTITY><<<(unsigned)blocks, threads, 0, stream>>>(in, eta, n, b, rp, t.l, sp);
  else {
    set_error("segmented solve supports the identity and cross-stencil right-hand sides");
    return NTK_ERR_UNSUPPORTED;
  }
  int rc = cuda_status(cudaGetLastError(), "seg_fwd_kernel");
  if (rc) return rc;
  seg_bwd_kernel<<<(unsigned)blocks, threads, 0, stream>>>(eta, out, n, b, t.g, t.w, sp);
  return cuda_status(cudaGetLastError(), "seg_bwd_kernel");
}

}  // namespace ntk
