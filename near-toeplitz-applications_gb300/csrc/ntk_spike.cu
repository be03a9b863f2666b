// ntk_spike.cu -- FP32 solve + double-word refinement for long systems
// whose LU multipliers decay too slowly for overlapping windows.
//
// The windows of ntk_long_refine.cu and ntk_adi_refine.cu truncate the
// coupling between a window and the rest of its system, which is exact to
// rounding only where the LU multipliers' products fall below 2^-56 within
// the halo.  Here nothing is truncated.  A system of n rows is cut into P
// partitions of 512 rows (the last one padded with identity rows), one warp
// each, and the FP32 solve is the exact partitioned solve of the reference's
// distributed algorithm (parallelcompact/reduced.py:135-196, sum.py:8-31,
// misc.py:21-46), on one GPU with the partitions of a system in one CTA:
//
//   A_p y_p = d_p       each partition's block with its coupling removed
//                       (a = 0 in its first row, c = 0 in its last row),
//                       solved by the warp's chunked FP32 LU (exact lane
//                       scans, no decay assumed);
//   R z = g             the reduced system of the 2(P - 1) end unknowns
//                       L_p (last row of partition p) and F_p (first row of
//                       partition p): g holds the y_p end values and
//                       R = I + the spikes' end values;
//   x_p = y_p - L_{p-1} v_p - F_{p+1} w_p
//                       with the spikes v_p = a(first row) A_p^-1 e_first
//                       and w_p = c(last row) A_p^-1 e_last.
//
// The spikes and R^-1 depend on the matrix only: they are computed once per
// plan in FP64 on the host and kept in FP32.  The end rows of every
// partition take the reduced solution's values, so the owning warp and its
// neighbour use bit-identical values there, and the residual d - A x (exact,
// in double-word FP32, of the full matrix) sees a consistent x.  Refinement
// sweeps then work as in ntk_refine.cuh: each FP32 solve has an error of
// about cond(A) 2^-24, each sweep multiplies the error by about that factor,
// down to a floor set by the residual's accuracy.  The matrices this path
// serves are the badly conditioned ones, so the residual is formed from the
// exact 53-bit right-hand side with exact products and compensated sums
// (residual_exact), which keeps that floor at the double-word's precision
// instead of cond(A) times it, and the last correction is added in FP64 so
// the result carries a full double's precision.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ntk_refine.cuh"
#include "ntk_spike.h"

namespace ntk {
namespace spike_detail {

using namespace refine_detail;

constexpr int M = 16;        // rows per lane
constexpr int PW = 32 * M;   // rows per partition (one warp)
constexpr int CP = class_pitch4<M>();

struct SpikeArgs {
  int n = 0, P = 0, R = 0;      // rows, partitions, reduced unknowns 2 (P - 1)
  const float4* tab = nullptr;  // distinct lane tables (ChunkTabs layout), CP float4s each
  const int* cls = nullptr;     // [P][32]: offset (float4s) of each lane's table
  const float2* spk = nullptr;  // [P][PW]: (v_p, w_p) per row
  const float* rinv = nullptr;  // [R][R]: R^-1, row-major
  DW ai, bi, ci;                // interior rows
  int nh = 1, nt = 1;           // special rows at the head / tail
  DW hd[2][3], td[2][3];        // their (a, b, c), double-word; td[nt - 1] is row n - 1
  float i3[3], hd3[2][3], td3[2][3];  // the coefficients' third words (coef = h + l + third exactly)
  unsigned* status = nullptr;   // bit 0: input outside the double-word range
};

// The FP32 solve of the whole system: x holds this warp's partition of the
// RHS and receives its part of the solution.  xl, xr receive the solution
// at the rows just before and after the partition (0 at the system's ends),
// which equal the neighbouring warps' own values bit for bit.  gz: 2R floats
// of shared memory.  Every thread of the CTA calls it (two CTA barriers).
__device__ __forceinline__ void global_solve(float (&x)[M], const ChunkTabs& t, const SpikeArgs& a, int p,
                                             unsigned lane, float* gz, float& xl, float& xr) {
  chunk_solve<M, false>(x, t, lane);
  const int P = a.P, R = a.R;
  float* g = gz;
  float* z = gz + R;
  if (lane == 31 && p < P - 1) g[2 * p] = x[M - 1];
  if (lane == 0 && p > 0) g[2 * p - 1] = x[0];
  __syncthreads();
  const int tid = threadIdx.x;
  if (tid < R) {
    const float* row = a.rinv + tid * R;
    float acc = 0.f;
    for (int c = 0; c < R; ++c) acc = fmaf(__ldg(row + c), g[c], acc);
    z[tid] = acc;
  }
  __syncthreads();
  const float Lm = p > 0 ? z[2 * p - 2] : 0.f;
  const float Fp = p < P - 1 ? z[2 * p + 1] : 0.f;
  const float4* sp = reinterpret_cast<const float4*>(a.spk + (size_t)p * PW + lane * M);
#pragma unroll
  for (int k = 0; k < M; k += 2) {
    const float4 s = __ldg(sp + k / 2);
    x[k] = fmaf(-Fp, s.y, fmaf(-Lm, s.x, x[k]));
    x[k + 1] = fmaf(-Fp, s.w, fmaf(-Lm, s.z, x[k + 1]));
  }
  if (lane == 0 && p > 0) x[0] = z[2 * p - 1];
  if (lane == 31 && p < P - 1) x[M - 1] = z[2 * p];
  xl = Lm;
  xr = Fp;
}

// The last 6 bits of x's 53-bit significand (what split_f64's hi and lo do
// not hold) as an exact float: x = hi + lo + third_word(x).  Zero below
// 2^-74 (where the float would be subnormal) and wherever lo is dropped.
__device__ __forceinline__ float third_word(double x) {
  const unsigned h = (unsigned)__double2hiint(x);
  const unsigned l = (unsigned)__double2loint(x);
  const unsigned mag = h & 0x7fffffffu;
  const unsigned hb = __funnelshift_l(l, h - (896u << 20), 3);
  // bits l[5:0] as an exact float integer, weight 2^(e - 1075)
  const float t = __fsub_rn(__uint_as_float((l & 63u) | 0x4b000000u), 8388608.0f);
  const float sc = __uint_as_float((hb & 0x7f800000u) - (52u << 23));
  const float v = __uint_as_float(__float_as_uint(__fmul_rn(t, sc)) | (h & 0x80000000u));
  return (mag >= (949u << 20) && mag < (1151u << 20)) ? v : 0.0f;
}

// r = D - (a x_m + b x_0 + c x_p) for D = dh + dl + d3 (the exact FP64
// right-hand side) and x = xh + xl, with every product split exactly
// (TwoProd) and every low-order term accumulated in a compensated
// double-word.  The plain double-word residual of ntk_refine.cuh rounds its
// low-order sum at ~2^-48 |A||x|, which the solve amplifies by cond(A): about
// 1e-12 for the ADI matrix at r = 40.  Here the rounding is ~2^-24 |r| plus
// ~2^-70 |A||x|, so the refinement reaches the double-word's own precision.
__device__ __forceinline__ float residual_exact(float dh, float dl, float d3, float xm, float x0, float xp, float lm,
                                                float l0, float lp, DW ca, DW cb, DW cc, float a3, float b3,
                                                float c3) {
  float pa, ea, pb, eb, pc, ec;
  two_prod(ca.h, xm, pa, ea);
  two_prod(cb.h, x0, pb, eb);
  two_prod(cc.h, xp, pc, ec);
  float s, es, p, ep;
  two_sum(pa, pc, s, es);
  two_sum(pb, s, p, ep);
  float h, eh;
  two_sum(dh, -p, h, eh);  // dh - p = h + eh exactly
  float T = dl, t = d3;
  auto add = [&](float v) {
    float u, e;
    two_sum(T, v, u, e);
    T = u;
    t += e;
  };
  auto addp = [&](float c, float v) {  // -(c v), exactly
    float q, e;
    two_prod(c, v, q, e);
    add(-q);
    t -= e;
  };
  add(eh);
  add(-ep);
  add(-es);
  add(-ea);
  add(-eb);
  add(-ec);
  addp(ca.h, lm);
  addp(cb.h, l0);
  addp(cc.h, lp);
  addp(ca.l, xm);
  addp(cb.l, x0);
  addp(cc.l, xp);
  t -= fmaf(ca.l, lm, fmaf(cb.l, l0, cc.l * lp));
  t -= fmaf(a3, xm, fmaf(b3, x0, c3 * xp));
  float r, er;
  two_sum(h, T, r, er);
  return r + (er + t);
}

// x + d as a normalised double-word (h, e), e also collecting xl
__device__ __forceinline__ void accumulate(float x, float d, float xl, float& h, float& e) {
  float s, t;
  two_sum(x, d, s, t);
  t += xl;
  fast_two_sum(s, t, h, e);
}

// One system per CTA, one warp per partition (blockDim = 32 P).
template <int SWEEPS>
__global__ void __launch_bounds__(32 * SPIKE_MAX_PARTS) spike_kernel(const double* in, double* out, Batch b,
                                                                   SpikeArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int SP = sys_pitch<M>();
  double* tiles = reinterpret_cast<double*>(smem_raw);                // [P][SP]: FP64 in, (hi, lo) of the RHS
  float* third = reinterpret_cast<float*>(tiles + (size_t)a.P * SP);  // [P][SP]: the RHS's third word
  float* gz = third + (size_t)a.P * SP;
  const int p = threadIdx.x >> 5;
  const unsigned lane = threadIdx.x & 31;
  const int j = lane;
  float* d3row = third + (size_t)p * SP;
  const long long off = sys_offset(blockIdx.x, b);
  const int n = a.n;
  const int pr0 = p * PW;
  double* trow = tiles + (size_t)p * SP;
  float2* drow = reinterpret_cast<float2*>(trow);
  // stage the partition (lanes walk rows), rows beyond n as zeros
#pragma unroll 4
  for (int q = 0; q < M; ++q) {
    const int i = j + 32 * q;
    const int r = pr0 + i;
    trow[tile_off<M>(i)] = r < n ? in[off + (long long)r * b.es] : 0.0;
  }
  __syncwarp();
  const int cb = j * (M + 1);
  const int r0 = pr0 + j * M;  // this lane's first row
  unsigned range = 0;
  float x[M];
#pragma unroll
  for (int k = 0; k < M; ++k) {
    float h, l;
    const double dv = trow[cb + k];
    split_f64(dv, h, l, range);
    x[k] = h;
    drow[cb + k] = make_float2(h, l);
    if (SWEEPS > 0) d3row[cb + k] = third_word(dv);
  }
  ChunkTabs tabs;
  tabs.q = a.tab + __ldg(a.cls + p * 32 + j);
  float nbl, nbr;  // solution at rows pr0 - 1 and pr0 + PW
  global_solve(x, tabs, a, p, lane, gz, nbl, nbr);
  float xl[M];
#pragma unroll
  for (int k = 0; k < M; ++k) xl[k] = 0.f;
  float nbl_l = 0.f, nbr_l = 0.f;  // their low parts
#pragma unroll
  for (int sweep = 0; sweep < SWEEPS; ++sweep) {
    float xleft = __shfl_up_sync(FULL, x[M - 1], 1);
    float xright = __shfl_down_sync(FULL, x[0], 1);
    float lleft = __shfl_up_sync(FULL, xl[M - 1], 1);
    float lright = __shfl_down_sync(FULL, xl[0], 1);
    if (j == 0) {
      xleft = nbl;
      lleft = nbl_l;
    }
    if (j == 31) {
      xright = nbr;
      lright = nbr_l;
    }
    float r[M];
#pragma unroll
    for (int k = 0; k < M; ++k) {
      const float2 d = drow[cb + k];
      const float xm = (k == 0) ? xleft : x[k - (k > 0)];
      const float xp = (k == M - 1) ? xright : x[k + (k < M - 1)];
      const float lm = (k == 0) ? lleft : xl[k - (k > 0)];
      const float lp = (k == M - 1) ? lright : xl[k + (k < M - 1)];
      r[k] = residual_exact(d.x, d.y, d3row[cb + k], xm, x[k], xp, lm, xl[k], lp, a.ai, a.bi, a.ci, a.i3[0],
                            a.i3[1], a.i3[2]);
      if (r0 + k >= n) r[k] = 0.f;  // padding rows
    }
    // head rows (partition 0, lane 0, rows 0 and 1)
    if (p == 0 && j == 0) {
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        if (k < a.nh) {
          const float2 d = drow[cb + k];
          const float xm = (k == 0) ? 0.f : x[0];
          const float lm = (k == 0) ? 0.f : xl[0];
          r[k] = residual_exact(d.x, d.y, d3row[cb + k], xm, x[k], x[k + 1], lm, xl[k], xl[k + 1], a.hd[k][0],
                                a.hd[k][1], a.hd[k][2], a.hd3[k][0], a.hd3[k][1], a.hd3[k][2]);
        }
      }
    }
    // tail rows n - nt .. n - 1: every row position is tested (compile-time
    // positions keep x and xl in registers)
    if (r0 + M > n - a.nt && r0 < n) {
#pragma unroll
      for (int k = 0; k < M; ++k) {
        const int ti = r0 + k - (n - a.nt);  // 0 .. nt-1 for the tail rows
        if (ti >= 0 && ti < a.nt) {
          const bool last = (r0 + k == n - 1);
          const float2 d = drow[cb + k];
          const float xm = (k == 0) ? xleft : x[k - (k > 0)];
          const float lm = (k == 0) ? lleft : xl[k - (k > 0)];
          const float xp = last ? 0.f : (k == M - 1) ? xright : x[k + (k < M - 1)];
          const float lp = last ? 0.f : (k == M - 1) ? lright : xl[k + (k < M - 1)];
          const DW ta = ti == 0 ? a.td[0][0] : a.td[1][0];
          const DW tb = ti == 0 ? a.td[0][1] : a.td[1][1];
          const DW tc = ti == 0 ? a.td[0][2] : a.td[1][2];
          const float ta3 = ti == 0 ? a.td3[0][0] : a.td3[1][0];
          const float tb3 = ti == 0 ? a.td3[0][1] : a.td3[1][1];
          const float tc3 = ti == 0 ? a.td3[0][2] : a.td3[1][2];
          r[k] = residual_exact(d.x, d.y, d3row[cb + k], xm, x[k], xp, lm, xl[k], lp, ta, tb, tc, ta3, tb3, tc3);
        }
      }
    }
    float dl, dr;
    global_solve(r, tabs, a, p, lane, gz, dl, dr);
    if (sweep + 1 < SWEEPS) {
#pragma unroll
      for (int k = 0; k < M; ++k) accumulate(x[k], r[k], xl[k], x[k], xl[k]);
      accumulate(nbl, dl, nbl_l, nbl, nbl_l);
      accumulate(nbr, dr, nbr_l, nbr, nbr_l);
    } else {
      // x + xl + delta summed in FP64: all 53 bits of the result (a
      // double-word would keep 47, and the ADI step's next stencil
      // amplifies that rounding by about cond(A))
#pragma unroll
      for (int k = 0; k < M; ++k) trow[cb + k] = __dadd_rn(__dadd_rn((double)x[k], (double)xl[k]), (double)r[k]);
    }
  }
  if (SWEEPS == 0) {
#pragma unroll
    for (int k = 0; k < M; ++k) trow[cb + k] = (double)x[k];
  }
  if (range && a.status) atomicOr(a.status, 1u);
  __syncwarp();
#pragma unroll 4
  for (int q = 0; q < M; ++q) {
    const int i = j + 32 * q;
    const int r = pr0 + i;
    if (r < n) out[off + (long long)r * b.es] = trow[tile_off<M>(i)];
  }
}

size_t spike_smem(int P) {
  return (size_t)P * sys_pitch<M>() * (sizeof(double) + sizeof(float)) +
         (size_t)4 * (P > 1 ? P - 1 : 1) * sizeof(float);
}

}  // namespace spike_detail

struct SpikeSolver {
  int n = 0, P = 0, R = 0, sweeps = 1;
  float4* d_tab = nullptr;
  int* d_cls = nullptr;
  float2* d_spk = nullptr;
  float* d_rinv = nullptr;
  unsigned* d_status = nullptr;
  spike_detail::SpikeArgs args;
  ~SpikeSolver() {
    if (d_tab) cudaFree(d_tab);
    if (d_cls) cudaFree(d_cls);
    if (d_spk) cudaFree(d_spk);
    if (d_rinv) cudaFree(d_rinv);
    if (d_status) cudaFree(d_status);
  }
};

namespace {

DW to_dw(double v) {
  DW d;
  d.h = (float)v;
  d.l = (float)(v - (double)d.h);
  return d;
}
// what to_dw(v) leaves out (exact: the 53-bit v needs at most 72 bits)
float third(double v) {
  const DW d = to_dw(v);
  return (float)((v - (double)d.h) - (double)d.l);
}

template <class T>
int upload(T** dst, const std::vector<T>& v, const char* what) {
  int rc = cuda_status(cudaMalloc(dst, sizeof(T) * v.size()), what);
  if (!rc) rc = cuda_status(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice), what);
  return rc;
}

}  // namespace

int spike_create(SpikeSolver** out, const Matrix& m, int sweeps) {
  using namespace spike_detail;
  *out = nullptr;
  const int n = m.n;
  const int P = (n + PW - 1) / PW;
  if (P < 2 || P > SPIKE_MAX_PARTS) {
    set_error("partitioned FP32 solve: need 512 < n <= %d (got %d)", SPIKE_MAX_PARTS * PW, n);
    return NTK_ERR_UNSUPPORTED;
  }
  if (sweeps < 0 || sweeps > 2) {
    set_error("FP32/refine with slowly decaying LU factors: at most 2 refinement sweeps (got %d)", sweeps);
    return NTK_ERR_UNSUPPORTED;
  }
  const int R = 2 * (P - 1);
  // the partitions' blocks, their FP64 LU, lane tables and spikes
  std::vector<std::vector<float>> lanes((size_t)P * 32, std::vector<float>(4 * (size_t)CP, 0.f));
  std::vector<float2> spk((size_t)P * PW, make_float2(0.f, 0.f));
  std::vector<double> vend(P, 0.0), vbeg(P, 0.0), wend(P, 0.0), wbeg(P, 0.0);
  for (int p = 0; p < P; ++p) {
    const int pr0 = p * PW;
    std::vector<double> aa(PW, 0.0), bb(PW, 1.0), cc(PW, 0.0);
    for (int i = 0; i < PW; ++i) {
      const int r = pr0 + i;
      if (r >= n) break;
      aa[i] = m.a(r);
      bb[i] = m.b(r);
      cc[i] = m.c(r);
    }
    const double ca = aa[0], cl = cc[PW - 1];  // coupling to the neighbouring partitions
    aa[0] = 0.0;
    cc[PW - 1] = 0.0;
    std::vector<double> l(PW, 0.0), u(PW, 0.0);
    u[0] = bb[0];
    for (int i = 1; i < PW; ++i) {
      l[i] = aa[i] / u[i - 1];
      u[i] = bb[i] - l[i] * cc[i - 1];
    }
    for (int i = 0; i < PW; ++i)
      if (!(std::fabs(u[i]) > 0.0) || !std::isfinite(u[i]) || !std::isfinite(l[i])) {
        set_error("partitioned FP32 solve: partition %d of the matrix is singular without pivoting", p);
        return NTK_ERR_UNSUPPORTED;
      }
    auto solve = [&](const std::vector<double>& d) {
      std::vector<double> y(PW), x(PW);
      y[0] = d[0];
      for (int i = 1; i < PW; ++i) y[i] = d[i] - l[i] * y[i - 1];
      x[PW - 1] = y[PW - 1] / u[PW - 1];
      for (int i = PW - 2; i >= 0; --i) x[i] = (y[i] - cc[i] * x[i + 1]) / u[i];
      return x;
    };
    if (p > 0) {
      std::vector<double> e(PW, 0.0);
      e[0] = 1.0;
      std::vector<double> v = solve(e);
      for (int i = 0; i < PW; ++i) spk[(size_t)p * PW + i].x = (float)(ca * v[i]);
      vbeg[p] = ca * v[0];
      vend[p] = ca * v[PW - 1];
    }
    if (p < P - 1) {
      std::vector<double> e(PW, 0.0);
      e[PW - 1] = 1.0;
      std::vector<double> w = solve(e);
      for (int i = 0; i < PW; ++i) spk[(size_t)p * PW + i].y = (float)(cl * w[i]);
      wbeg[p] = cl * w[0];
      wend[p] = cl * w[PW - 1];
    }
    // lane tables (ChunkTabs: per group of four rows the float4s L, G, W, PHI, PSI)
    for (int j = 0; j < 32; ++j) {
      std::vector<float>& t = lanes[(size_t)p * 32 + j];
      double phi = 1.0, psi = 1.0;
      std::vector<double> ph(M), ps(M);
      for (int k = 0; k < M; ++k) {
        phi *= -l[j * M + k];
        ph[k] = phi;
      }
      for (int k = M - 1; k >= 0; --k) {
        const int i = j * M + k;
        psi *= -(cc[i] / u[i]);
        ps[k] = psi;
      }
      for (int k = 0; k < M; ++k) {
        const int i = j * M + k;
        float* grp = t.data() + 4 * (5 * (k / 4));
        const int e = k % 4;
        grp[0 * 4 + e] = (float)l[i];
        grp[1 * 4 + e] = (float)(1.0 / u[i]);
        grp[2 * 4 + e] = (float)(cc[i] / u[i]);
        grp[3 * 4 + e] = (float)ph[k];
        grp[4 * 4 + e] = (float)ps[k];
      }
    }
  }
  // reduced system R z = g: z[2p] = L_p (p <= P-2), z[2p-1] = F_p (p >= 1)
  std::vector<double> Rm((size_t)R * R, 0.0), Ri((size_t)R * R, 0.0);
  for (int i = 0; i < R; ++i) Rm[(size_t)i * R + i] = 1.0;
  for (int p = 0; p < P; ++p) {
    const int rows[2] = {2 * p, 2 * p - 1};  // L_p, F_p equations
    for (int q = 0; q < 2; ++q) {
      const int row = rows[q];
      if (row < 0 || row >= R || (q == 0 && p > P - 2)) continue;
      if (p > 0) Rm[(size_t)row * R + 2 * p - 2] += q == 0 ? vend[p] : vbeg[p];
      if (p < P - 1) Rm[(size_t)row * R + 2 * p + 1] += q == 0 ? wend[p] : wbeg[p];
    }
  }
  {
    // Gauss-Jordan with partial pivoting
    std::vector<double> A(Rm);
    for (int i = 0; i < R; ++i) Ri[(size_t)i * R + i] = 1.0;
    double amax = 0.0;
    for (double v : A) amax = std::max(amax, std::fabs(v));
    for (int c = 0; c < R; ++c) {
      int piv = c;
      for (int i = c + 1; i < R; ++i)
        if (std::fabs(A[(size_t)i * R + c]) > std::fabs(A[(size_t)piv * R + c])) piv = i;
      if (!(std::fabs(A[(size_t)piv * R + c]) > 1e-12 * amax)) {
        set_error("partitioned FP32 solve: the reduced system is singular");
        return NTK_ERR_UNSUPPORTED;
      }
      if (piv != c)
        for (int k = 0; k < R; ++k) {
          std::swap(A[(size_t)piv * R + k], A[(size_t)c * R + k]);
          std::swap(Ri[(size_t)piv * R + k], Ri[(size_t)c * R + k]);
        }
      const double inv = 1.0 / A[(size_t)c * R + c];
      for (int k = 0; k < R; ++k) {
        A[(size_t)c * R + k] *= inv;
        Ri[(size_t)c * R + k] *= inv;
      }
      for (int i = 0; i < R; ++i) {
        if (i == c) continue;
        const double f = A[(size_t)i * R + c];
        if (f == 0.0) continue;
        for (int k = 0; k < R; ++k) {
          A[(size_t)i * R + k] -= f * A[(size_t)c * R + k];
          Ri[(size_t)i * R + k] -= f * Ri[(size_t)c * R + k];
        }
      }
    }
  }
  // distinct lane tables
  std::vector<int> rep, cls((size_t)P * 32);
  for (size_t q = 0; q < lanes.size(); ++q) {
    int c = -1;
    for (size_t k = 0; k < rep.size() && c < 0; ++k)
      if (std::memcmp(lanes[rep[k]].data(), lanes[q].data(), sizeof(float) * 4 * CP) == 0) c = (int)k;
    if (c < 0) {
      c = (int)rep.size();
      rep.push_back((int)q);
    }
    cls[q] = c * CP;
  }
  std::vector<float4> tab(rep.size() * (size_t)CP);
  for (size_t c = 0; c < rep.size(); ++c) std::memcpy(&tab[c * CP], lanes[rep[c]].data(), sizeof(float4) * CP);
  std::vector<float> rinv(Ri.size());
  for (size_t i = 0; i < Ri.size(); ++i) rinv[i] = (float)Ri[i];

  SpikeSolver* s = new (std::nothrow) SpikeSolver();
  if (!s) {
    set_error("out of host memory");
    return NTK_ERR_ALLOC;
  }
  s->n = n;
  s->P = P;
  s->R = R;
  s->sweeps = sweeps;
  int rc = upload(&s->d_tab, tab, "cudaMalloc/cudaMemcpy(partition tables)");
  if (!rc) rc = upload(&s->d_cls, cls, "cudaMalloc/cudaMemcpy(partition lane map)");
  if (!rc) rc = upload(&s->d_spk, spk, "cudaMalloc/cudaMemcpy(spikes)");
  if (!rc) rc = upload(&s->d_rinv, rinv, "cudaMalloc/cudaMemcpy(reduced inverse)");
  if (!rc) rc = cuda_status(cudaMalloc(&s->d_status, sizeof(unsigned)), "cudaMalloc(status)");
  if (!rc) rc = cuda_status(cudaMemset(s->d_status, 0, sizeof(unsigned)), "cudaMemset(status)");
  if (rc) {
    delete s;
    return rc;
  }
  SpikeArgs& a = s->args;
  a.n = n;
  a.P = P;
  a.R = R;
  a.tab = s->d_tab;
  a.cls = s->d_cls;
  a.spk = s->d_spk;
  a.rinv = s->d_rinv;
  a.ai = to_dw(m.ai);
  a.bi = to_dw(m.bi);
  a.ci = to_dw(m.ci);
  a.i3[0] = third(m.ai);
  a.i3[1] = third(m.bi);
  a.i3[2] = third(m.ci);
  a.nh = m.nh;
  a.nt = m.nt;
  for (int i = 0; i < 2; ++i) {
    const int hr = i, tr = n - m.nt + i;
    const double h3[3] = {hr == 0 ? 0.0 : m.a(hr), m.b(hr), m.c(hr)};
    const bool ok = i < m.nt;
    const double t3[3] = {ok ? m.a(tr) : 0.0, ok ? m.b(tr) : 1.0, ok && tr < n - 1 ? m.c(tr) : 0.0};
    for (int q = 0; q < 3; ++q) {
      a.hd[i][q] = to_dw(h3[q]);
      a.hd3[i][q] = third(h3[q]);
      a.td[i][q] = to_dw(t3[q]);
      a.td3[i][q] = third(t3[q]);
    }
  }
  a.status = s->d_status;
  *out = s;
  return NTK_OK;
}

void spike_destroy(SpikeSolver* s) { delete s; }

int spike_partitions(const SpikeSolver* s) { return s ? s->P : 0; }
int spike_sweeps(const SpikeSolver* s) { return s ? s->sweeps : 0; }

void spike_status_words(const SpikeSolver* s, std::vector<unsigned*>& out) {
  if (s && s->d_status) out.push_back(s->d_status);
}

int spike_solve(SpikeSolver* s, const double* in, double* out, const Batch& b, cudaStream_t st) {
  using namespace spike_detail;
  if (b.nsys <= 0) return NTK_OK;
  if (b.nsys > 0x7fffffffLL) {
    set_error("too many systems for one launch");
    return NTK_ERR_INVALID;
  }
  const size_t smem = spike_smem(s->P);
  auto pick = [&](auto kern) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_status(e, "cudaFuncSetAttribute(spike_kernel)");
    kern<<<(unsigned)b.nsys, 32 * s->P, smem, st>>>(in, out, b, s->args);
    return cuda_status(cudaGetLastError(), "spike_kernel");
  };
  switch (s->sweeps) {
    case 0: return pick(spike_kernel<0>);
    case 1: return pick(spike_kernel<1>);
    default: return pick(spike_kernel<2>);
  }
}

}  // namespace ntk
