// ntk_r2_group.cuh -- the per-group solves of the paired-chunk kernels
// (ntk_r2.cu, ntk_r2_adi.cu): given each thread's RHS high parts in
// registers and the (hi, lo) pairs in shared memory, the FP32 solve, the
// double-word residual, the FP32 correction solve and the FP64 output.
#pragma once
#include "ntk_r2_tma.cuh"

namespace ntk {
namespace r2 {

// ---------------------------------------------------------------------------
// contiguous systems: one warp per system, chunk carries by shuffles
// ---------------------------------------------------------------------------
// Offset (in doubles) of rows 2i, 2i+1 of chunk j in a 4 KB system tile
// written by TMA with the 128-byte swizzle is xpair(j, i) (ntk_r2_tma.cuh).
// The solve of one contiguous system by its warp (lane j owns chunk j):
// v[k] = (row k, row k + 8) of the chunk's RHS high parts in, hl the
// system's (hi, lo) RHS pairs in the swizzled layout (xpair), and the FP64
// results handed to store(i, row 2i, row 2i + 1, row 2i + 8, row 2i + 9).
// GEN: interior coefficients of any value (res_pair_gen).
// With GEN the constants live in shared memory: a compiler fence between the
// phases keeps their loads inside the phase that uses them (fewer registers
// live at once).
template <bool ON>
__device__ __forceinline__ void phase_fence() {
  if (ON) asm volatile("" ::: "memory");
}
template <int SWEEPS, bool GEN = false, class STORE>
__device__ __forceinline__ void contiguous_solve(float2 (&v)[8], const double* hl, int j, const Args& a,
                                                 STORE store) {
  const Consts& K = a.k;
  // ---- FP32 solve ----
  {
    float CA = __shfl_up_sync(FULL, fwd_local(v, K), 1);
    if (j == 0) CA = 0.f;
    bwd_local(v, CA, K);
    float XB = __shfl_down_sync(FULL, start_comb(v, K), 1);
    if (j == 31) XB = 0.f;
    bwd_fix(v, XB, K);
    if (j == 0) head_fix(v, K);
    if (j == 31) tail_fix(v, K);
  }
  if (SWEEPS == 0) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      double oa0, ob0, oa1, ob1;
      out_pair0(v[2 * i], a, oa0, ob0);
      out_pair0(v[2 * i + 1], a, oa1, ob1);
      store(i, oa0, oa1, ob0, ob1);
    }
  } else {
    phase_fence<GEN>();
    // ---- residual ----
    float xl = __shfl_up_sync(FULL, v[7].y, 1);
    float xr = __shfl_down_sync(FULL, v[0].x, 1);
    if (j == 0) xl = 0.f;
    if (j == 31) xr = 0.f;
    // the special rows' residuals (patched in after the interior ones)
    float rsp[2] = {0.f, 0.f};
    if (j == 0) {
#pragma unroll
      for (int q = 0; q < 2; ++q)
        if (q < a.nh) {
          const float2 d = reinterpret_cast<const float2*>(hl + xpair(0, 0))[q];
          rsp[q] = res_row(d.x, d.y, q == 0 ? 0.f : v[q - 1].x, v[q].x, v[q + 1].x, a.hd[q][0], a.hd[q][1],
                           a.hd[q][2]);
        }
    }
    if (j == 31) {
#pragma unroll
      for (int q = 0; q < 2; ++q)
        if (q < a.nt) {
          const int k = 7 - q;  // row n-1-q is B[k] of the last chunk
          const float2 d = reinterpret_cast<const float2*>(hl + xpair(31, (8 + k) >> 1))[(8 + k) & 1];
          const int ti = a.nt - 1 - q;
          rsp[q] = res_row(d.x, d.y, v[k - 1].y, v[k].y, q == 0 ? 0.f : v[k + 1].y, a.td[ti][0], a.td[ti][1],
                           a.td[ti][2]);
        }
    }
    float2 r[8];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float4 qa = *reinterpret_cast<const float4*>(hl + xpair(j, i));
      const float4 qb = *reinterpret_cast<const float4*>(hl + xpair(j, i + 4));
      const int k0 = 2 * i, k1 = 2 * i + 1;
      const float2 xm0 = (k0 == 0) ? pair(xl, v[7].x) : v[k0 - 1];
      r[k0] = res_interior<GEN>(pair(qa.x, qb.x), pair(qa.y, qb.y), xm0, v[k0], v[k0 + 1], a);
      const float2 xp1 = (k1 == 7) ? pair(v[0].y, xr) : v[k1 + 1];
      r[k1] = res_interior<GEN>(pair(qa.z, qb.z), pair(qa.w, qb.w), v[k1 - 1], v[k1], xp1, a);
    }
    if (j == 0) {
      if (a.nh > 0) r[0].x = rsp[0];
      if (a.nh > 1) r[1].x = rsp[1];
    }
    if (j == 31) {
      if (a.nt > 0) r[7].y = rsp[0];
      if (a.nt > 1) r[6].y = rsp[1];
    }
    phase_fence<GEN>();
    // ---- FP32 correction solve ----
    float CA = __shfl_up_sync(FULL, fwd_local(r, K), 1);
    if (j == 0) CA = 0.f;
    bwd_local(r, CA, K);
    float XB = __shfl_down_sync(FULL, start_comb(r, K), 1);
    if (j == 31) XB = 0.f;
    bwd_fix(r, XB, K);
    if (j == 0) head_fix(r, K);
    if (j == 31) tail_fix(r, K);
    phase_fence<GEN>();
    // ---- s (x + delta) as FP64 ----
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      double oa0, ob0, oa1, ob1;
      out_pair(v[2 * i], r[2 * i], a, oa0, ob0);
      out_pair(v[2 * i + 1], r[2 * i + 1], a, oa1, ob1);
      store(i, oa0, oa1, ob0, ob1);
    }
  }
}

// ---------------------------------------------------------------------------
// strided systems: 16 systems per group, thread (s, c) = system s, chunk c;
// chunk carries and edge values through shared memory with group barriers
// ---------------------------------------------------------------------------
constexpr int SG = 16;  // systems per group (128 contiguous bytes per row)
// exchange arrays, [chunk][system] floats each
enum { X_E1 = 0, X_S1, X_A0, X_B0, X_B7, X_E2, X_S2, X_COUNT };

// The solve of one strided system's chunk by thread (s, c) of a 16-system
// group: v[k] = (row k, row k + 8) of the chunk's RHS high parts in; col
// points at the system's row 0 in a tile of PITCH doubles per row whose
// slots of this chunk's rows hold the (hi, lo) RHS pairs (read by the
// residual); after_first() runs after the first barrier (every halo row of
// the RHS has been read then); the FP64 results go to store(k, value) for
// row 16 c + k.
template <int SWEEPS, int PITCH, class SYNC, class AFTER, class STORE>
__device__ __forceinline__ void strided_solve(float2 (&v)[8], double* col, float* xch, int s, int c, const Args& a,
                                              SYNC sync, AFTER after_first, STORE store) {
  const int r0 = ROWS * c;
  auto X = [&](int which, int chunk) -> float& { return xch[(which * CHUNKS + chunk) * SG + s]; };
  const Consts& K = a.k;
  // ---- FP32 solve ----
  X(X_E1, c) = fwd_local(v, K);
  sync();  // carries published; every halo row has been read
  after_first();
  bwd_local(v, c > 0 ? X(X_E1, c - 1) : 0.f, K);
  const float S1 = start_comb(v, K);
  X(X_S1, c) = S1;
  X(X_A0, c) = v[0].x;
  X(X_B0, c) = v[0].y;
  X(X_B7, c) = v[7].y;
  sync();
  bwd_fix(v, c < CHUNKS - 1 ? X(X_S1, c + 1) : 0.f, K);
  if (c == 0) head_fix(v, K);
  if (c == CHUNKS - 1) tail_fix(v, K);
  if (SWEEPS == 0) {
#pragma unroll
    for (int k = 0; k < HALF; ++k) {
      double oa, ob;
      out_pair0(v[k], a, oa, ob);
      store(k, oa);
      store(k + HALF, ob);
    }
    return;
  }
  // ---- residual ----
  const float xl = c > 0 ? left_edge(X(X_B7, c - 1), S1, K) : 0.f;
  const float xr =
      c < CHUNKS - 1 ? right_edge(X(X_A0, c + 1), X(X_B0, c + 1), c + 2 < CHUNKS ? X(X_S1, c + 2) : 0.f, K) : 0.f;
  // the special rows' residuals (patched in after the interior ones)
  float rsp[2] = {0.f, 0.f};
  if (c == 0) {
#pragma unroll
    for (int q = 0; q < 2; ++q)
      if (q < a.nh) {
        const float2 d = reinterpret_cast<const float2*>(col + q * PITCH)[0];
        rsp[q] =
            res_row(d.x, d.y, q == 0 ? 0.f : v[q - 1].x, v[q].x, v[q + 1].x, a.hd[q][0], a.hd[q][1], a.hd[q][2]);
      }
  }
  if (c == CHUNKS - 1) {
#pragma unroll
    for (int q = 0; q < 2; ++q)
      if (q < a.nt) {
        const int k = HALF - 1 - q;
        const float2 d = reinterpret_cast<const float2*>(col + (r0 + HALF + k) * PITCH)[0];
        const int ti = a.nt - 1 - q;
        rsp[q] = res_row(d.x, d.y, v[k - 1].y, v[k].y, q == 0 ? 0.f : v[k + 1].y, a.td[ti][0], a.td[ti][1],
                         a.td[ti][2]);
      }
  }
  float2 r[8];
#pragma unroll
  for (int k = 0; k < HALF; ++k) {
    const float2 da = reinterpret_cast<const float2*>(col + (r0 + k) * PITCH)[0];
    const float2 db = reinterpret_cast<const float2*>(col + (r0 + k + HALF) * PITCH)[0];
    const float2 xm = (k == 0) ? pair(xl, v[HALF - 1].x) : v[k - 1];
    const float2 xp = (k == HALF - 1) ? pair(v[0].y, xr) : v[k + 1];
    r[k] = res_pair(pair(da.x, db.x), pair(da.y, db.y), xm, v[k], xp, a);
  }
  if (c == 0) {
    if (a.nh > 0) r[0].x = rsp[0];
    if (a.nh > 1) r[1].x = rsp[1];
  }
  if (c == CHUNKS - 1) {
    if (a.nt > 0) r[HALF - 1].y = rsp[0];
    if (a.nt > 1) r[HALF - 2].y = rsp[1];
  }
  // ---- FP32 correction solve ----
  X(X_E2, c) = fwd_local(r, K);
  sync();
  bwd_local(r, c > 0 ? X(X_E2, c - 1) : 0.f, K);
  X(X_S2, c) = start_comb(r, K);
  sync();
  bwd_fix(r, c < CHUNKS - 1 ? X(X_S2, c + 1) : 0.f, K);
  if (c == 0) head_fix(r, K);
  if (c == CHUNKS - 1) tail_fix(r, K);
#pragma unroll
  for (int k = 0; k < HALF; ++k) {
    double oa, ob;
    out_pair(v[k], r[k], a, oa, ob);
    store(k, oa);
    store(k + HALF, ob);
  }
}

}  // namespace r2
}  // namespace ntk
