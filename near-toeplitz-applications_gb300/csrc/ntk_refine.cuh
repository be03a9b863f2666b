// ntk_refine.cuh -- FP32 chunked solve + double-word iterative refinement.
//
// Replaces the same reference path as ntk_solve_f64.cu (the cyclic
// reduction of neato.py:8-124, with compact/rhs.py:9-37 fused in) for the
// precisions NTK_FP32 and NTK_FP32_REFINE.
//
// Why this shape on GB300.  HBM delivers ~6.7 TB/s = ~420 G rows/s at 16 B
// per row, ~1.45 rows per clock per SM.  The FP64 pipe retires ~1.7
// instructions per clock per SM, so the plain FP64 solve (4 FP64
// instructions per row) tops out near 30% of HBM.  Here the FP64 pipe is used
// once per row (the DADD that forms the compact RHS difference f_{i+1} -
// f_{i-1} exactly as the FP64 path does) and everything else runs on the
// FP32/INT pipes:
//   * the FP64 difference is split into a float pair with integer operations;
//   * the residual r = d - A x and the accumulation of the correction use
//     error-free transformations (TwoSum/TwoProd), so they carry ~48
//     significant bits -- what an FP64 residual would supply for a 1e-12
//     result (the FP32 solve leaves ~5e-7, one sweep ~(5e-7)^2 * cond);
//   * the FP32 solves run on register-resident chunks;
//   * the FP64 output is assembled from the double-word with integer
//     operations (dw_to_f64).
//
// Work decomposition.  A CTA stages W systems into shared memory with
// coalesced loads (contiguous systems: lanes walk rows; strided y/z systems:
// lanes walk adjacent systems, so no permute pass is needed).  One warp
// solves one system, lane j owning rows [j*M, (j+1)*M).  The solve applies
// the shared matrix's LU factors (FP64 on the host, rounded to FP32)
// chunk-wise: each lane runs the forward and backward recurrences over its
// chunk from zero and the chunk-to-chunk carries of both first-order linear
// recurrences are resolved with 5-step warp-shuffle scans.  The staged tile
// uses a padded layout (chunk pitch M+1, system pitch 32(M+1)+1 words), so
// both the staging accesses and the per-lane chunk accesses are free of bank
// conflicts; after the RHS is formed, each tile slot holds that row's
// double-word RHS (two floats) for the residual sweeps.  Rows whose
// coefficients differ from the interior ones (the matrix's boundary rows and
// the compact scheme's one-sided boundary stencils) are computed in FP64 by
// the lane that owns them.
#pragma once
#include <cstdio>

#include "ntk_device.cuh"
#include "ntk_internal.h"
#include "ntk_plan.h"

namespace ntk {

struct DW {
  float h, l;
};

struct RefineArgs {
  // FP32 factor tables per lane class: lanes whose chunks see identical
  // factors share one table (typically three classes: the first chunk, the
  // interior chunks, the chunk holding row n-1).  Layout: [class of each
  // lane: 32 ints] [class tables: ncls x class_pitch4 float4s, see
  // ChunkTabs].  (The lane map lives in device memory: indexing a kernel
  // parameter by lane would force a local copy of the whole parameter
  // block.)
  const float* tab = nullptr;
  int ncls = 32;
  DW ai, bi, ci;               // interior row coefficients
  int nh = 1, nt = 1;          // special rows: head 0..nh-1, tail n-nt..n-1
  DW hd[2][3];                 // head rows (a, b, c), double-word
  DW td[2][3];                 // tail rows (a, b, c), double-word; td[nt-1] is row n-1
  double sigma0 = 1.0, sigmaN = 1.0;  // compact boundary RHS scales
  DW s;                               // output scale x = s * xi
  int unit_scale = 1;
  unsigned* status = nullptr;  // bit 0: input outside the FP32+refine range
};

template <int M, bool DECAY, int SPW>
int refine_dispatch(const double* in, double* out, int n, const Batch& b, const RefineArgs& ra, bool pow2,
                    int sweeps, int rhs, int W, cudaStream_t st);

// The plan's FP32 state for callers outside ntk_refine.cu (the ADI windows):
// kernel arguments for right-hand-side scales sigma0/sigmaN and output scale
// s, and the kernel shape (rows per lane, power-of-two interior, one-shuffle
// carries).
int refine_args(const Plan& p, double sigma0, double sigmaN, double s, RefineArgs* ra, int* M, bool* pow2,
                bool* decay);

// RHS kind of refine_system for tiles that already hold the double-word RHS
// (hi, lo) in their slots (the ADI windows form their stencil themselves).
constexpr int RHS_PRESPLIT = 100;

namespace refine_detail {

constexpr unsigned FULL = 0xffffffffu;

template <int M>
__host__ __device__ constexpr int sys_pitch() {
  return 32 * (M + 1) + 1;
}
// Pitch of the system tiles of a group of S strided systems (S a power of
// two): a half-warp of the staging map below touches S systems times 16 / S
// adjacent rows; a pitch of 16 / S (mod 16 doubles) puts those 16 eight-byte
// words in 16 different bank pairs.  Rows within a tile keep the chunk pitch
// M + 1, so the solves' own accesses are unaffected.
// Unit-stride groups are copied one system per warp and keep sys_pitch
// (measured 1-2% faster there).
template <int M>
__host__ __device__ constexpr int group_pitch(int S, long long es) {
  return es == 1 ? sys_pitch<M>() : 32 * (M + 1) + (S < 16 ? 16 / S : 1);
}
template <int M>
__device__ __forceinline__ int tile_off(int r) {
  return (r / M) * (M + 1) + (r % M);
}

// Per-row FP32 tables of one lane's chunk, in groups of four rows so one
// 16-byte shared-memory load serves four rows: group j (rows 4j..4j+3) is
// five float4s
//   L[j]    forward multipliers l_i
//   G[j]    g_i = 1/u_i
//   Wv[j]   w_i = c_i/u_i
//   PHI[j]  phi_i = prod_{chunk start..i} (-l)
//   PSI[j]  psi_i = prod_{i..chunk end} (-w)
// phi and psi are the responses of a chunk's local sweeps to the carry that
// enters it; they depend only on the row position, so they are tabulated
// once per plan instead of being recomputed (and held in registers) per row.
template <int M>
__host__ __device__ constexpr int class_pitch4() {
  return 5 * (M / 4) + 1;  // float4s per lane class (+1: classes start on different banks)
}
struct ChunkTabs {
  const float4* q;  // this lane's class: 5 float4s per group of four rows
};
__device__ __forceinline__ float comp4(const float4& v, int c) {
  return c == 0 ? v.x : c == 1 ? v.y : c == 2 ? v.z : v.w;
}

// The table loads of a fully unrolled sweep would otherwise all be hoisted
// to its start; a compiler-only fence per group of four rows bounds how far
// ahead they are issued.
#define NTK_TABLE_FENCE(k) \
  if (((k) & 3) == 3) asm volatile("" ::: "memory")

// FP32 chunked LU solve, in place on v (RHS in, solution out).
// DECAY: the factor products over every chunk (prod |l|, prod |w| over M
// rows) are below 2^-26, i.e. below FP32 rounding, so the carry entering a
// chunk is the previous chunk's local end value alone and the carry scans
// reduce to one shuffle each (the plan checks the products on the host).
template <int M, bool DECAY>
__device__ __forceinline__ void chunk_solve(float (&v)[M], const ChunkTabs& t, unsigned lane) {
  static_assert(M % 4 == 0, "rows per lane must be a multiple of 4");
  float yh = 0.f;
  float4 L4;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    if ((k & 3) == 0) L4 = t.q[5 * (k >> 2) + 0];
    yh = fmaf(-comp4(L4, k & 3), yh, v[k]);
    v[k] = yh;
    NTK_TABLE_FENCE(k);
  }
  float B = yh;
  if (!DECAY) {
    float A = t.q[5 * (M / 4 - 1) + 3].w;  // phi of the chunk's last row
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const float Ap = __shfl_up_sync(FULL, A, d);
      const float Bp = __shfl_up_sync(FULL, B, d);
      if (lane >= (unsigned)d) {
        B = fmaf(A, Bp, B);
        A = A * Ap;
      }
    }
  }
  float Yprev = __shfl_up_sync(FULL, B, 1);
  if (lane == 0) Yprev = 0.f;
  float xh = 0.f;
  float4 G4, W4, P4;
#pragma unroll
  for (int k = M - 1; k >= 0; --k) {
    if ((k & 3) == 3) {
      G4 = t.q[5 * (k >> 2) + 1];
      W4 = t.q[5 * (k >> 2) + 2];
      P4 = t.q[5 * (k >> 2) + 3];
    }
    const float y = fmaf(comp4(P4, k & 3), Yprev, v[k]);
    xh = fmaf(-comp4(W4, k & 3), xh, comp4(G4, k & 3) * y);
    v[k] = xh;
    if ((k & 3) == 0) asm volatile("" ::: "memory");
  }
  float B2 = xh;
  if (!DECAY) {
    float A2 = t.q[4].x;  // psi of the chunk's first row
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const float Ap = __shfl_down_sync(FULL, A2, d);
      const float Bp = __shfl_down_sync(FULL, B2, d);
      if (lane + d < 32u) {
        B2 = fmaf(A2, Bp, B2);
        A2 = A2 * Ap;
      }
    }
  }
  float Xnext = __shfl_down_sync(FULL, B2, 1);
  if (lane == 31) Xnext = 0.f;
  float4 S4;
#pragma unroll
  for (int k = 0; k < M; ++k) {
    if ((k & 3) == 0) S4 = t.q[5 * (k >> 2) + 4];
    v[k] = fmaf(comp4(S4, k & 3), Xnext, v[k]);
    NTK_TABLE_FENCE(k);
  }
}

// r = D - A*x for one interior row, x = xh (+ xl).  A*xh is formed as an
// exact double-word p + ep: the products are exact (power-of-two
// coefficients) or split with TwoProd, and are summed with TwoSum.  dh - p is
// then exact whenever it cancels (Sterbenz: dh and p within a factor of 2),
// and otherwise its rounding is relative to r itself, so no third TwoSum is
// needed; the low-order terms are collected in the tail.
template <bool POW2, bool HASLO>
__device__ __forceinline__ float residual_row(float dh, float dl, float xm, float x0, float xp, float lm, float l0,
                                              float lp, DW ca, DW cb, DW cc) {
  float pa, pb, pc, ea = 0.f, eb = 0.f, ec = 0.f;
  if (POW2) {
    pa = __fmul_rn(ca.h, xm);
    pb = __fmul_rn(cb.h, x0);
    pc = __fmul_rn(cc.h, xp);
  } else {
    two_prod(ca.h, xm, pa, ea);
    two_prod(cb.h, x0, pb, eb);
    two_prod(cc.h, xp, pc, ec);
  }
  float s, es, p, ep;
  two_sum(pa, pc, s, es);
  two_sum(pb, s, p, ep);
  float tail = __fsub_rn(dl, __fadd_rn(ep, es));
  if (!POW2) {
    tail -= (ea + eb) + ec;
    tail -= fmaf(ca.l, xm, fmaf(cb.l, x0, cc.l * xp));
  }
  if (HASLO) tail -= fmaf(ca.h, lm, fmaf(cb.h, l0, cc.h * lp));
  return __fadd_rn(__fsub_rn(dh, p), tail);
}

#ifndef NTK_REFINE_OCC
#define NTK_REFINE_OCC 3
#endif
template <int M>
struct RefineOcc {
  static constexpr int value = (M <= 16) ? NTK_REFINE_OCC : 1;
};
// Launch bounds of refine_kernel.  "wide" variants fit 64 registers with at
// most a few words of spill (rows per lane <= 8, or 16 rows with one system
// per warp and at most one sweep): 32 resident warps per SM and CTAs of up to
// 16 warps (measured on GB300 for 512-row systems: 4% faster unit-stride and
// 6% faster strided than 24 warps at 80 registers).  Two sweeps spill
// 120-290 bytes at 64 registers; two systems per warp spill 30-80 bytes there
// and measured no faster.  Both keep 80 registers and CTAs of up to 8 warps.
template <int M, int SWEEPS, int SPW>
struct RefineShape {
  static constexpr bool wide = (M <= 8 || (M == 16 && SPW == 1 && SWEEPS <= 1));
  static constexpr int max_threads = wide ? 512 : 256;
  static constexpr int min_blocks = wide ? 2 : RefineOcc<M>::value;
};
// A CTA stages at most 16 systems (the first warp's lanes 2s, 2s + 1 form the
// boundary rows of system s).
constexpr int REFINE_MAX_GROUP = 16;

// Shared-memory footprint of one CTA: S padded system tiles, the class
// tables (class_pitch4 float4s per class), and the boundary stencils'
// inputs (3 doubles) and double-word results for rows 0 and n-1 of each
// system.
template <int M>
__host__ __device__ constexpr size_t refine_smem(int S, int ncls, long long es) {
  return (((size_t)S * group_pitch<M>(S, es) * sizeof(double) + 15) & ~(size_t)15) +
         (size_t)ncls * class_pitch4<M>() * sizeof(float4) + (size_t)2 * S * (sizeof(float2) + 3 * sizeof(double));
}

// Offset of system s's first unknown: (s / ni) * os + (s % ni) * is, with
// 32-bit division whenever the operands allow.
__device__ __forceinline__ long long sys_offset(long long s, const Batch& b) {
  if (b.ni >= b.nsys) return s * b.is;
  if (s <= 0x7fffffffLL && b.ni <= 0x7fffffffLL) {
    const unsigned q = (unsigned)s / (unsigned)b.ni;
    const unsigned r = (unsigned)s - q * (unsigned)b.ni;
    return (long long)q * b.os + (long long)r * b.is;
  }
  return (s / b.ni) * b.os + (s % b.ni) * b.is;
}

// x = s * (h + l) as an FP64 value (no FP64 instruction)
template <class ARGS>
__device__ __forceinline__ double scaled_out(float h, float l, const ARGS& ra) {
  if (!ra.unit_scale) {
    float p, e, oh, ol;
    two_prod(ra.s.h, h, p, e);
    e = fmaf(ra.s.h, l, e);
    e = fmaf(ra.s.l, h, e);
    fast_two_sum(p, e, oh, ol);
    return dw_to_f64(oh, ol);
  }
  return dw_to_f64(h, l);
}

// s * (x + d) for an FP32 solution x and its FP32 correction d, as an FP64
// value: s_h * x is split exactly (TwoProd) and the small terms s_h * d and
// s_l * x are added to its error (s_l * d lies below the double-word's
// precision), then the pair is normalised and assembled.
template <class ARGS>
__device__ __forceinline__ double corrected_out(float x, float d, const ARGS& ra) {
  float h, e;
  if (ra.unit_scale) {
    two_sum(x, d, h, e);
  } else {
    const float p = __fmul_rn(ra.s.h, x);
    float t = __fmaf_rn(ra.s.h, x, -p);
    t = __fmaf_rn(ra.s.h, d, t);
    t = __fmaf_rn(ra.s.l, x, t);
    fast_two_sum(p, t, h, e);
  }
  return dw_to_f64(h, e);
}

// One system, solved by one warp in place in its padded tile trow: RHS
// (bndw: the double-word right-hand sides of rows 0 and n-1), FP32 solve,
// refinement sweeps; the FP64 result is left in the tile slots.
// ARGS: RefineArgs, or any type with the same row-coefficient fields (ai, bi,
// ci, nh, nt, hd, td) and output scale (s, unit_scale).
template <int M, int RHS, int SWEEPS, bool POW2, bool PAD, bool DECAY, class ARGS = RefineArgs>
__device__ __forceinline__ void refine_system(double* trow, const float2* bndw, const ChunkTabs& tabs, int n,
                                              const ARGS& ra, unsigned lane, unsigned& range) {
  const int j = lane;
  const int r0 = j * M;
  const int cb = j * (M + 1);  // this lane's chunk in the tile
  float2* drow = reinterpret_cast<float2*>(trow);
  const int n1 = n - 1;
  const bool tail_here = (r0 <= n1) && (n1 < r0 + M);  // owns row n-1
  float x[M];

  // ---- RHS in double-word, written back into the tile slots ----
  if (RHS == RHS_COMPACT) {
    // D_r = f_{r+1} - f_{r-1} is formed in FP64 (one DADD, as in the FP64
    // path) and then split: a double-word split of f itself keeps only
    // ~2^-47 |f|, too coarse when f_{r+1} and f_{r-1} nearly cancel.  Rows 0
    // and n-1 take the boundary stencils staged in bnd.
    const double fleft = (j > 0) ? trow[tile_off<M>(r0 - 1)] : 0.0;
    const double fright = (j < 31) ? trow[tile_off<M>(r0 + M)] : 0.0;
    __syncwarp();  // the neighbours' halo reads happen before any slot is rewritten
    double fprev = fleft, fcur = trow[cb];
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const double fnext = (k < M - 1) ? trow[cb + k + 1] : fright;
      float h, l;
      split_f64(fnext - fprev, h, l, range);  // h: D truncated to FP32, l: the next 23 bits
      x[k] = h;
      drow[cb + k] = make_float2(h, l);
      fprev = fcur;
      fcur = fnext;
    }
    if (j == 0) {
      const float2 d0 = bndw[0];
      x[0] = d0.x;
      drow[cb + 0] = d0;
    }
    if (tail_here) {
      const float2 d1 = bndw[1];
      const float h = d1.x;
      if (!PAD) {
        x[M - 1] = h;
      } else {
#pragma unroll
        for (int k = 0; k < M; ++k)
          if (r0 + k == n1) x[k] = h;
      }
      drow[tile_off<M>(n1)] = d1;
    }
  } else if (RHS == RHS_PRESPLIT) {
#pragma unroll
    for (int k = 0; k < M; ++k) x[k] = drow[cb + k].x;
  } else {
#pragma unroll
    for (int k = 0; k < M; ++k) {
      float h, l;
      split_f64(trow[cb + k], h, l, range);  // h: d truncated to FP32, l: the next 23 bits
      x[k] = h;
      drow[cb + k] = make_float2(h, l);
    }
  }

  // ---- FP32 solve ----
  chunk_solve<M, DECAY>(x, tabs, lane);

  // ---- refinement sweeps; the last one writes the FP64 result ----
  float xl[M];
#pragma unroll
  for (int k = 0; k < M; ++k) xl[k] = 0.f;
  if (SWEEPS == 0) {
#pragma unroll
    for (int k = 0; k < M; ++k) trow[cb + k] = scaled_out(x[k], 0.f, ra);
  }
#pragma unroll
  for (int sweep = 0; sweep < SWEEPS; ++sweep) {
    // every lane executes every shuffle (full mask); edges are zeroed after
    float xleft = __shfl_up_sync(FULL, x[M - 1], 1);
    float xright = __shfl_down_sync(FULL, x[0], 1);
    if (j == 0) xleft = 0.f;
    if (j == 31) xright = 0.f;
    float lleft = 0.f, lright = 0.f;
    if (sweep > 0) {  // sweep is warp-uniform
      lleft = __shfl_up_sync(FULL, xl[M - 1], 1);
      lright = __shfl_down_sync(FULL, xl[0], 1);
      if (j == 0) lleft = 0.f;
      if (j == 31) lright = 0.f;
    }
    float r[M];
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const float2 d = drow[cb + k];
      const float xm = (k == 0) ? xleft : x[k - (k > 0)];
      const float xp = (k == M - 1) ? xright : x[k + (k < M - 1)];
      if (sweep == 0) {
        r[k] = residual_row<POW2, false>(d.x, d.y, xm, x[k], xp, 0.f, 0.f, 0.f, ra.ai, ra.bi, ra.ci);
      } else {
        const float lm = (k == 0) ? lleft : xl[k - (k > 0)];
        const float lp = (k == M - 1) ? lright : xl[k + (k < M - 1)];
        r[k] = residual_row<POW2, true>(d.x, d.y, xm, x[k], xp, lm, xl[k], lp, ra.ai, ra.bi, ra.ci);
      }
    }
    // rows with their own coefficients, in double-word FP32 like the
    // interior: head rows sit in lane 0 at compile-time positions
    if (j == 0) {
#pragma unroll
      for (int k = 0; k < 2 && k < M; ++k) {
        if (k < ra.nh) {
          const float2 d = drow[cb + k];
          const float xm = (k == 0) ? 0.f : x[k - (k > 0)];
          const float lm = (k == 0) ? 0.f : xl[k - (k > 0)];
          const float xp = (k == M - 1) ? xright : x[k + (k < M - 1)];
          const float lp = (k == M - 1) ? lright : xl[k + (k < M - 1)];
          r[k] = residual_row<false, true>(d.x, d.y, xm, x[k], xp, lm, xl[k], lp, ra.hd[k][0], ra.hd[k][1],
                                           ra.hd[k][2]);
        }
      }
    }
    // tail rows
    if (r0 + M > n - ra.nt && r0 < n) {
      if (!PAD) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int k = M - 1 - q;  // row n-1-q
          if (q < ra.nt && k >= 0) {
            const int ti = ra.nt - 1 - q;
            const float2 d = drow[cb + k];
            const float xm = (k == 0) ? xleft : x[k - (k > 0)];
            const float lm = (k == 0) ? lleft : xl[k - (k > 0)];
            const float xp = (q == 0) ? 0.f : x[k + (k < M - 1)];
            const float lp = (q == 0) ? 0.f : xl[k + (k < M - 1)];
            r[k] = residual_row<false, true>(d.x, d.y, xm, x[k], xp, lm, xl[k], lp, ra.td[ti][0], ra.td[ti][1],
                                             ra.td[ti][2]);
          }
        }
      } else {
        // runtime position: gather the needed values with selects
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int row = n1 - q;
          if (q < ra.nt && row >= r0 && row < r0 + M) {
            const int kk = row - r0;
            float xh0 = 0.f, xl0 = 0.f, xhm = 0.f, xlm = 0.f, xhp = 0.f, xlp = 0.f;
#pragma unroll
            for (int k = 0; k < M; ++k) {
              if (k == kk) {
                xh0 = x[k];
                xl0 = xl[k];
              }
              if (k == kk - 1) {
                xhm = x[k];
                xlm = xl[k];
              }
              if (k == kk + 1) {
                xhp = x[k];
                xlp = xl[k];
              }
            }
            if (kk == 0) {
              xhm = xleft;
              xlm = lleft;
            }
            if (kk == M - 1) {
              xhp = xright;
              xlp = lright;
            }
            if (q == 0) {
              xhp = 0.f;
              xlp = 0.f;
            }
            const int ti = ra.nt - 1 - q;
            const float2 d = drow[tile_off<M>(row)];
            const float rr = residual_row<false, true>(d.x, d.y, xhm, xh0, xhp, xlm, xl0, xlp, ra.td[ti][0],
                                                       ra.td[ti][1], ra.td[ti][2]);
#pragma unroll
            for (int k = 0; k < M; ++k)
              if (k == kk) r[k] = rr;
          }
        }
      }
    }
    chunk_solve<M, DECAY>(r, tabs, lane);
    if (sweep + 1 < SWEEPS) {
      // x + delta as a normalised double-word for the next sweep
#pragma unroll
      for (int k = 0; k < M; ++k) {
        float h, e;
        two_sum(x[k], r[k], h, e);
        e += xl[k];
        fast_two_sum(h, e, x[k], xl[k]);
      }
    } else {
      // last sweep: s * (x + delta) straight to the FP64 output slot
#pragma unroll
      for (int k = 0; k < M; ++k) {
        if (sweep == 0) {
          trow[cb + k] = corrected_out(x[k], r[k], ra);
        } else {
          float h, e;
          two_sum(x[k], r[k], h, e);
          e += xl[k];
          fast_two_sum(h, e, h, e);
          trow[cb + k] = scaled_out(h, e, ra);
        }
      }
    }
  }
}

// ---- staging map ----
// A CTA of W warps stages S = SPW * W systems (SPW systems per warp).
// Contiguous systems (es == 1): warp w copies its systems w + kW, lanes
// walking rows (256-byte rows of copies).  Strided systems: lanes walk the S
// adjacent systems (S * 8-byte segments per row), thread t taking system
// t % S and rows t / S + RS q, RS = 32 W / S rows per step.  Slot of row r:
// tile_off(r); for a step of RS rows the slot advances by (RS / M)(M + 1).
// The same thread stores the same rows at the end.
__device__ __forceinline__ int group_count(const Batch& b, long long grp, int S) {
  const long long left = b.nsys - grp * S;
  return (int)(left < S ? left : S);
}

template <int M, int SPW, bool PAD>
__device__ __forceinline__ void refine_copy(const double* in, double* out, double* tiles, int n, const Batch& b,
                                            long long grp, int W, bool load) {
  const int S = SPW * W;
  const int P = group_pitch<M>(S, b.es);
  const int wc = group_count(b, grp, S);
  if (b.es == 1) {
    constexpr int QSTEP = (32 / M) * (M + 1);
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < SPW; ++k) {
      const int sw = (int)(threadIdx.x >> 5) + k * W;
      if (sw < wc) {
        const long long off = sys_offset(grp * S + sw, b) + lane;
        double* tslot = tiles + (size_t)sw * P + tile_off<M>(lane);
#pragma unroll
        for (int q = 0; q < M; ++q) {
          const bool ok = !PAD || lane + 32 * q < n;
          if (load)
            cp_async8(tslot + q * QSTEP, ok ? in + off + 32 * q : in, ok ? 8u : 0u);
          else if (ok)
            out[off + 32 * q] = tslot[q * QSTEP];
        }
      }
    }
  } else {
    constexpr int RS = 32 / SPW;  // rows per step (blockDim / S)
    static_assert(RS % M == 0, "rows per step must be a multiple of the rows per lane");
    constexpr int QSTEP = (RS / M) * (M + 1);
    const int sw = (int)threadIdx.x % S;
    const int rb = (int)threadIdx.x / S;
    if (sw < wc) {
      const long long gstep = (long long)RS * b.es;
      long long off = sys_offset(grp * S + sw, b) + (long long)rb * b.es;
      double* tslot = tiles + (size_t)sw * P + tile_off<M>(rb);
      // the address is advanced step by step (q * gstep offsets would be held
      // in registers)
#pragma unroll
      for (int q = 0; q < M * SPW; ++q) {
        const bool ok = !PAD || rb + RS * q < n;
        if (load)
          cp_async8(tslot + q * QSTEP, ok ? in + off : in, ok ? 8u : 0u);
        else if (ok)
          out[off] = tslot[q * QSTEP];
        off += gstep;
      }
    }
  }
}

// One group of S systems per CTA: stage (cp.async, all copies in flight at
// once), CTA barrier, each warp solves its SPW systems, CTA barrier, store.
// The compact scheme's one-sided boundary stencils (compact/rhs.py:21-31)
// are evaluated in FP64 for all S systems by the first warp (lane 2s: row 0
// of system s, lane 2s+1: row n-1) from their own small copies: one set of
// FP64 instructions per CTA instead of one per system.
template <int M, int RHS, int SWEEPS, bool POW2, bool PAD, bool DECAY, int SPW>
__global__ void __launch_bounds__(RefineShape<M, SWEEPS, SPW>::max_threads,
                                  RefineShape<M, SWEEPS, SPW>::min_blocks)
    refine_kernel(const double* in, double* out, int n, Batch b, RefineArgs ra) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int W = blockDim.x >> 5;
  const int S = SPW * W;
  const int P = group_pitch<M>(S, b.es);
  const int TC = ra.ncls * class_pitch4<M>();  // table float4s
  double* tiles = reinterpret_cast<double*>(smem_raw);  // [S][P]
  float4* tq = reinterpret_cast<float4*>(smem_raw + (((size_t)S * P * sizeof(double) + 15) & ~(size_t)15));
  float2* bnd = reinterpret_cast<float2*>(tq + TC);    // [2S]: rows 0, n-1
  double* braw = reinterpret_cast<double*>(bnd + 2 * S);  // [2S][3]: stencil inputs
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const unsigned lane = tid & 31;
  const long long grp = blockIdx.x;
  const int wc = group_count(b, grp, S);
  unsigned range = 0;

  const int cbase = __ldg(reinterpret_cast<const int*>(ra.tab) + lane) * class_pitch4<M>();
  {
    const float4* g4 = reinterpret_cast<const float4*>(ra.tab + 32);
    for (int i = tid; i < TC; i += blockDim.x) tq[i] = g4[i];
  }
  refine_copy<M, SPW, PAD>(in, nullptr, tiles, n, b, grp, W, true);
  if (RHS == RHS_COMPACT && warp == 0 && (int)(lane >> 1) < wc) {
    const bool tl = lane & 1;
    const double* f = in + sys_offset(grp * S + (lane >> 1), b);
    const long long e = b.es;
    double* dst = braw + (size_t)lane * 3;
    cp_async8(dst + 0, f + (tl ? (long long)(n - 1) * e : 0), 8u);
    cp_async8(dst + 1, f + (tl ? (long long)(n - 2) * e : e), 8u);
    cp_async8(dst + 2, f + (tl ? (long long)(n - 3) * e : 2 * e), 8u);
  }
  cp_async_wait_all();
  if (RHS == RHS_COMPACT && warp == 0) {
    __syncwarp();
    if ((int)(lane >> 1) < wc) {
      const double* r = braw + (size_t)lane * 3;
      const double v = ((lane & 1) ? ra.sigmaN : ra.sigma0) * ((-5.0 * r[0] + 4.0 * r[1]) + r[2]);
      float h, l;
      split_f64(v, h, l, range);
      fast_two_sum(h, l, h, l);
      bnd[lane] = make_float2(h, l);
    }
  }
  __syncthreads();  // group staged, boundary right-hand sides written
  ChunkTabs tabs;
  tabs.q = tq + cbase;
#pragma unroll
  for (int k = 0; k < SPW; ++k) {
    const int sys = warp + k * W;
    if (sys < wc)
      refine_system<M, RHS, SWEEPS, POW2, PAD, DECAY>(tiles + (size_t)sys * P, bnd + 2 * sys, tabs, n, ra, lane,
                                                      range);
  }
  __syncthreads();  // group solved: results in the tile slots
  refine_copy<M, SPW, PAD>(nullptr, out, tiles, n, b, grp, W, false);
  if (range && ra.status) atomicOr(ra.status, 1u);
}

template <int M, int RHS, int SWEEPS, bool POW2, bool PAD, bool DECAY, int SPW>
int launch_one(const double* in, double* out, int n, const Batch& b, const RefineArgs& ra, int W, cudaStream_t st) {
  // the widest CTA this variant is compiled for
  constexpr int WMAX = RefineShape<M, SWEEPS, SPW>::max_threads / 32 < REFINE_MAX_GROUP / SPW
                           ? RefineShape<M, SWEEPS, SPW>::max_threads / 32
                           : REFINE_MAX_GROUP / SPW;
  if (W > WMAX) W = WMAX;
  const int S = SPW * W;
  const size_t smem = refine_smem<M>(S, ra.ncls, b.es);
  auto kern = refine_kernel<M, RHS, SWEEPS, POW2, PAD, DECAY, SPW>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(refine_kernel)");
  const long long blocks = (b.nsys + S - 1) / S;
  if (blocks > 0x7fffffffLL) {
    set_error("too many systems for one launch");
    return NTK_ERR_INVALID;
  }
  kern<<<(unsigned)blocks, W * 32, smem, st>>>(in, out, n, b, ra);
  return cuda_status(cudaGetLastError(), "refine_kernel");
}

template <int M, int RHS, int SWEEPS, bool DECAY, int SPW>
int dispatch_pp(const double* in, double* out, int n, const Batch& b, const RefineArgs& ra, bool pow2, int W,
                cudaStream_t st) {
  const bool pad = (n != 32 * M);
  if (pow2)
    return pad ? launch_one<M, RHS, SWEEPS, true, true, DECAY, SPW>(in, out, n, b, ra, W, st)
               : launch_one<M, RHS, SWEEPS, true, false, DECAY, SPW>(in, out, n, b, ra, W, st);
  return pad ? launch_one<M, RHS, SWEEPS, false, true, DECAY, SPW>(in, out, n, b, ra, W, st)
             : launch_one<M, RHS, SWEEPS, false, false, DECAY, SPW>(in, out, n, b, ra, W, st);
}

template <int M, int RHS, bool DECAY, int SPW>
int dispatch_sweeps(const double* in, double* out, int n, const Batch& b, const RefineArgs& ra, bool pow2,
                    int sweeps, int W, cudaStream_t st) {
  switch (sweeps) {
    case 0: return dispatch_pp<M, RHS, 0, DECAY, SPW>(in, out, n, b, ra, pow2, W, st);
    case 1: return dispatch_pp<M, RHS, 1, DECAY, SPW>(in, out, n, b, ra, pow2, W, st);
    default: return dispatch_pp<M, RHS, 2, DECAY, SPW>(in, out, n, b, ra, pow2, W, st);
  }
}

}  // namespace refine_detail

// Kernel instances for one M, one carry mode (DECAY) and one number of
// systems per warp (SPW); the ntk_refine_m*.cu translation units
// instantiate them, ntk_refine.cu picks one.
template <int M, bool DECAY, int SPW>
int refine_dispatch(const double* in, double* out, int n, const Batch& b, const RefineArgs& ra, bool pow2,
                    int sweeps, int rhs, int W, cudaStream_t st) {
  using namespace refine_detail;
  if (rhs == RHS_COMPACT) return dispatch_sweeps<M, RHS_COMPACT, DECAY, SPW>(in, out, n, b, ra, pow2, sweeps, W, st);
  return dispatch_sweeps<M, RHS_IDENTITY, DECAY, SPW>(in, out, n, b, ra, pow2, sweeps, W, st);
}

}  // namespace ntk
