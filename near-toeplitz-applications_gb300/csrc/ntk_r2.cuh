// ntk_r2.cuh -- per-thread arithmetic of the paired-chunk FP32 + refinement
// solve for systems of 512 rows (kernels in ntk_r2.cu).  Every function here
// compiles for the device and for the host, so the host emulation of the
// kernels' data flow (tests/r2_emul.cpp) produces the GPU's results bit for
// bit.
//
// Replaces, for n = 512, the cyclic reduction of neato.py:8-124 with
// compact/rhs.py:9-37 fused in, like ntk_refine.cuh, with three changes that
// cut the instructions per row:
//
//  * One thread owns a 16-row chunk and holds it as 8 pairs (row k, row
//    k + 8): the two 8-row halves (sub-chunks A and B) run the recurrences
//    side by side in packed FP32x2 instructions (FFMA2 / FADD2 / FMUL2 issue
//    once for two rows on sm_100+), and the residual and output arithmetic,
//    which is independent per row, is packed the same way.
//  * The FP32 solve factors the pure Toeplitz matrix T (interior a, b, c,
//    T[0][0] = u_inf, the fixed point of the pivot recurrence), whose LU
//    factors are the same constants for every row: no per-row factor tables
//    (they are kernel parameters).  The matrix A differs from T in its first
//    nh and last nt rows only; the rank-(nh + nt) difference is applied with
//    the Sherman-Morrison-Woodbury formula, x = z - P C_h^-1 (delta^T z) at
//    the head and the same at the tail, where z = T^-1 d.  The correction
//    vectors T^-1 e_i decay like l^k, so the head correction touches the
//    first chunk only (rows 0..14) and the tail correction the last chunk
//    (rows 497..511); the truncation, below 2^-26 relative, is part of the
//    FP32 solve's error, which the refinement removes.
//  * The chunk carries of the two first-order recurrences are truncated
//    after two sub-chunks (16 rows): the plan only uses this solve when
//    l^16 and w^16 are below 2^-26.
//
// The residual r = d - A x (A's own rows, special head and tail rows
// included) is formed exactly in double-word FP32 (power-of-two interior
// coefficients: exact products, TwoSum, Sterbenz), as in ntk_refine.cuh.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define R2_HD __host__ __device__ __forceinline__
#else
#define R2_HD inline
#endif

namespace ntk {
namespace r2 {

constexpr int NROWS = 512;  // system length served by this solve
constexpr int ROWS = 16;    // rows per chunk (one thread)
constexpr int HALF = 8;     // rows per sub-chunk
constexpr int CHUNKS = 32;  // chunks per system

// ---------------------------------------------------------------------------
// bit casts and integer helpers
// ---------------------------------------------------------------------------
R2_HD unsigned f2u(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  unsigned u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
R2_HD float u2f(unsigned u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}
R2_HD unsigned dhi(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2hiint(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return (unsigned)(u >> 32);
#endif
}
R2_HD unsigned dlo(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned)__double2loint(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return (unsigned)u;
#endif
}
R2_HD double mkd(unsigned hi, unsigned lo) {
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t u = ((uint64_t)hi << 32) | lo;
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
R2_HD unsigned umax(unsigned a, unsigned b) { return a > b ? a : b; }
// (hi << 3) | (lo >> 29)
R2_HD unsigned shl3_funnel(unsigned lo, unsigned hi) {
#ifdef __CUDA_ARCH__
  return __funnelshift_l(lo, hi, 3);
#else
  return (hi << 3) | (lo >> 29);
#endif
}

// ---------------------------------------------------------------------------
// FP32 and FP64 arithmetic with explicit rounding (never contracted)
// ---------------------------------------------------------------------------
R2_HD float fma_(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
R2_HD float add_(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
R2_HD float mul_(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
R2_HD double dadd_(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
R2_HD double dsub_(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
R2_HD double dmul_(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
R2_HD double dfma_(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}

// packed pairs: one FFMA2 / FADD2 / FMUL2 instruction on sm_100+
R2_HD float2 ffma2(float2 a, float2 b, float2 c) {
#ifdef __CUDA_ARCH__
  return __ffma2_rn(a, b, c);
#else
  return make_float2(std::fmaf(a.x, b.x, c.x), std::fmaf(a.y, b.y, c.y));
#endif
}
R2_HD float2 fadd2(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
R2_HD float2 fmul2(float2 a, float2 b) {
#ifdef __CUDA_ARCH__
  return __fmul2_rn(a, b);
#else
  return make_float2(a.x * b.x, a.y * b.y);
#endif
}
// a - b, one rounding (an FMA with an exact product by -1)
R2_HD float2 fsub2(float2 a, float2 b) { return ffma2(b, make_float2(-1.f, -1.f), a); }
R2_HD float2 pair(float a, float b) { return make_float2(a, b); }
R2_HD float2 splat(float a) { return make_float2(a, a); }

// error-free transformations on pairs (Knuth's TwoSum; Dekker's FastTwoSum
// for |a| >= |b|)
R2_HD void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = fadd2(a, b);
  const float2 bb = fsub2(s, a);
  e = fadd2(fsub2(a, fsub2(s, bb)), fsub2(b, bb));
}
R2_HD void two_sum(float a, float b, float& s, float& e) {
  s = add_(a, b);
  const float bb = add_(s, -a);
  e = add_(add_(a, -add_(s, -bb)), add_(b, -bb));
}
R2_HD void fast_two_sum(float a, float b, float& s, float& e) {
  s = add_(a, b);
  e = add_(b, -add_(s, a * -1.f));
}

// ---------------------------------------------------------------------------
// FP64 <-> double-word with integer and FP32 operations only (the FP64 pipe
// and the double<->float conversions run at 1/64 of the FP32 rate on GB300)
// ---------------------------------------------------------------------------
// x = hi + lo: hi = x truncated to 24 significant bits, lo = the next 23
// bits (l[28:6] of the low word, an exact float integer via 2^23 + m,
// scaled by 2^(e - 46)).  |x| < 2^-126: hi is 0 or below 2^-146;
// |x| < 2^-80: lo = 0.  rmax collects |x|'s high word: >= 1151 << 20 means
// |x| >= 2^128, inf or nan (out of the double-word range).
R2_HD void split_f64(double x, float& hi, float& lo, unsigned& rmax) {
  const unsigned h = dhi(x), l = dlo(x);
  const unsigned mag = h & 0x7fffffffu;
  const unsigned sign = h - mag;
  rmax = umax(rmax, mag);
  const unsigned t1 = umax(mag, 896u << 20) - (896u << 20);
  hi = u2f(shl3_funnel(l, t1) + sign);
  const float t = add_(u2f(((l >> 6) & 0x007fffffu) | 0x4b000000u), -8388608.0f);
  const unsigned e2 = umax(mag, 942u << 20) * 8u - (942u << 23);  // exponent bits wrap: (e - 942) << 23
  lo = mul_(t, u2f((e2 & 0x7f800000u) | sign));
}

// hi + lo (normalised: |lo| <= ulp(hi) / 2) as a double.  lo counts units of
// 2^(e_hi - 46) (64 ulps of hi as a double): k = round(lo * 2^(46 - e_hi))
// lies within +-2^22, so adding 1.5 * 2^23 rounds it into a float's low
// mantissa bits, and 64 k is added to the 64-bit pattern of |hi|.  Below
// an exact power of two the double's ulp halves and k counts twice.
// Relative error <= 2^-47; |hi| < 2^-126 gives |result| < 2^-126.
R2_HD double dw_to_f64(float hi, float lo) {
  const unsigned bh = f2u(hi);
  const unsigned ah = bh & 0x7fffffffu;
  const unsigned sign = bh - ah;
  const unsigned eh = umax(ah & 0x7f800000u, 47u << 23);  // keeps the scale finite for zero / tiny hi
  const float sc = u2f((300u << 23) - eh + sign);         // 2^(46 - e_hi) with hi's sign
  const float t = fma_(lo, sc, 12582912.0f);
  int k = (int)(f2u(t) - 0x4b400000u);
  if ((ah & 0x007fffffu) == 0u) k += (k < 0 ? k : 0);
  unsigned dh = (ah >> 3) + (896u << 20);
  dh = (ah >= 0x00800000u) ? dh : 0u;
  const uint64_t m = (((uint64_t)dh << 32) | (uint64_t)(ah << 29)) + (uint64_t)((int64_t)k * 64);
  return mkd((unsigned)(m >> 32) + sign, (unsigned)m);
}

// ---------------------------------------------------------------------------
// kernel parameters
// ---------------------------------------------------------------------------
// The FP32 factorisation of the pure Toeplitz matrix T and the end
// corrections (pairs hold the same value twice unless noted).
struct Consts {
  float2 nl;       // -l, l = a / u_inf
  float2 g;        // 1 / u_inf
  float2 nw;       // -w, w = c / u_inf
  float2 phi[8];   // (-l)^(k+1): forward response of row k of a sub-chunk to the carry entering it
  float2 psi[8];   // (-w)^(8-k): backward response of row k to the carry entering at the sub-chunk's end
  // head: beta_j = sum_m hd[j][m] z_m (m = 0, 1, 2); x_r -= sum_j beta_j P[j](r), rows 0..14
  float hdel[2][3];
  float2 P[2][8];  // (P_j(k), P_j(k + 8)), P_j(15) = 0
  // tail: beta'_j = sum_m tdel[j][m] z_{509 + m}; x_r -= sum_j beta'_j Q[j](r), chunk rows 1..15
  float tdel[2][3];
  float2 Q[2][8];  // (Q_j(k), Q_j(k + 8)) over the last chunk, Q_j(0) = 0
  int nh, nt;      // head / tail rows of A that differ from T (0..2 each)
};

// A double-word coefficient (hi, lo).
struct DWc {
  float h, l;
};

struct Args {
  Consts k;
  float2 ca, cb, cc;  // interior coefficients of A (powers of two or zero), as pairs
  // interior coefficients of any value (res_pair_gen): their low parts and
  // negated high parts; the low parts are zero for powers of two
  float2 cal, cbl, ccl, nca, ncb, ncc;
  int nh, nt;         // special rows of A: head 0..nh-1, tail n-nt..n-1
  DWc hd[2][3];       // head rows (a, b, c), double-word
  DWc td[2][3];       // tail rows (a, b, c), td[nt-1] is row n-1
  double sigma0, sigmaN;  // compact boundary RHS scales
  float2 sh, sl, nsh, nsl;  // output scale s = sh + sl and its negation, as pairs
  int unit_scale;
  unsigned* status;
};

// ---------------------------------------------------------------------------
// the chunk solve (FP32), in place on v[k] = (row k, row k + 8)
// ---------------------------------------------------------------------------
// Forward sweep of both sub-chunks from zero: v[k] = (a_k, b_k).  Returns
// E = b_7 + phi_7 a_7, the chunk's end value without the carry entering it
// (its weight, (-l)^16, is below 2^-26).
R2_HD float fwd_local(float2 (&v)[8], const Consts& c) {
  float2 y = v[0];
#pragma unroll
  for (int k = 1; k < 8; ++k) {
    y = ffma2(c.nl, y, v[k]);
    v[k] = y;
  }
  return fma_(c.phi[7].x, v[7].x, v[7].y);
}
// Backward sweep with the forward carry folded in: y = (a, b) + phi (CA, CB),
// x_k = g y_k - w x_{k+1} from zero at each sub-chunk's end.  CA is the
// previous chunk's E (0 in the first chunk).  Leaves v[k] = (alpha_k, beta_k).
R2_HD void bwd_local(float2 (&v)[8], float CA, const Consts& c) {
  const float CB = fma_(c.phi[7].x, CA, v[7].x);
  const float2 C = pair(CA, CB);
  float2 x = fmul2(c.g, ffma2(c.phi[7], C, v[7]));
  v[7] = x;
#pragma unroll
  for (int k = 6; k >= 0; --k) {
    const float2 y = ffma2(c.phi[k], C, v[k]);
    x = ffma2(c.nw, x, fmul2(c.g, y));
    v[k] = x;
  }
}
// S = alpha_0 + psi_0 beta_0: the chunk's start value without the carry
// entering at its end.
R2_HD float start_comb(const float2 (&v)[8], const Consts& c) { return fma_(c.psi[0].x, v[0].y, v[0].x); }
// The carry entering sub-chunk B (XB, the next chunk's S; 0 in the last
// chunk) and through it sub-chunk A: x_k = (alpha_k, beta_k) + psi_k (XA, XB).
R2_HD float fix_xa(const float2 (&v)[8], float XB, const Consts& c) { return fma_(c.psi[0].x, XB, v[0].y); }
R2_HD void bwd_fix(float2 (&v)[8], float XB, const Consts& c) {
  const float2 X = pair(fix_xa(v, XB, c), XB);
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = ffma2(c.psi[k], X, v[k]);
}
// Woodbury corrections of the first and last chunks (z = T^-1 d in v).
R2_HD void head_fix(float2 (&v)[8], const Consts& c) {
  float b[2] = {0.f, 0.f};
#pragma unroll
  for (int j = 0; j < 2; ++j)
    if (j < c.nh) b[j] = fma_(c.hdel[j][2], v[2].x, fma_(c.hdel[j][1], v[1].x, mul_(c.hdel[j][0], v[0].x)));
#pragma unroll
  for (int j = 0; j < 2; ++j)
    if (j < c.nh) {
      const float2 nb = splat(-b[j]);
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = ffma2(nb, c.P[j][k], v[k]);
    }
}
R2_HD void tail_fix(float2 (&v)[8], const Consts& c) {
  float b[2] = {0.f, 0.f};
#pragma unroll
  for (int j = 0; j < 2; ++j)
    if (j < c.nt) b[j] = fma_(c.tdel[j][2], v[7].y, fma_(c.tdel[j][1], v[6].y, mul_(c.tdel[j][0], v[5].y)));
#pragma unroll
  for (int j = 0; j < 2; ++j)
    if (j < c.nt) {
      const float2 nb = splat(-b[j]);
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = ffma2(nb, c.Q[j][k], v[k]);
    }
}
// The final FP32 values of the neighbouring chunks' edge rows, recomputed
// from what those chunks publish (bit-identical to the owners' own values;
// the end corrections leave these rows alone): row 15 of the chunk before
// (its beta_7 and the carry it received, this chunk's S) and row 0 of the
// chunk after (its alpha_0, beta_0 and the S of the chunk after it).
R2_HD float left_edge(float beta7_prev, float S_own, const Consts& c) { return fma_(c.psi[7].y, S_own, beta7_prev); }
R2_HD float right_edge(float alpha0_next, float beta0_next, float S_next2, const Consts& c) {
  const float XA = fma_(c.psi[0].x, S_next2, beta0_next);
  return fma_(c.psi[0].x, XA, alpha0_next);
}

// ---------------------------------------------------------------------------
// residual and output
// ---------------------------------------------------------------------------
// r = (dh + dl) - (a xm + b x0 + c xp) for power-of-two a, b, c: exact
// products, TwoSum of the three, Sterbenz-exact dh - p where they cancel.
R2_HD float2 res_pair(float2 dh, float2 dl, float2 xm, float2 x0, float2 xp, const Args& a) {
  const float2 pa = fmul2(a.ca, xm), pb = fmul2(a.cb, x0), pc = fmul2(a.cc, xp);
  float2 s, es, p, ep;
  two_sum2(pa, pc, s, es);
  two_sum2(pb, s, p, ep);
  const float2 tail = fsub2(dl, fadd2(ep, es));
  return fadd2(fsub2(dh, p), tail);
}
// The same for interior coefficients of any value, each a double-word
// (hi + lo): the high parts' product errors from FMAs (exact), the low
// parts' products added into the tail.
R2_HD float2 res_pair_gen(float2 dh, float2 dl, float2 xm, float2 x0, float2 xp, const Args& a) {
  const float2 pa = fmul2(a.ca, xm), pb = fmul2(a.cb, x0), pc = fmul2(a.cc, xp);
  // minus the product errors: pa - ca xm etc., exact
  const float2 na = ffma2(a.nca, xm, pa), nb = ffma2(a.ncb, x0, pb), nc = ffma2(a.ncc, xp, pc);
  float2 s, es, p, ep;
  two_sum2(pa, pc, s, es);
  two_sum2(pb, s, p, ep);
  const float2 lo = ffma2(a.cal, xm, ffma2(a.cbl, x0, fmul2(a.ccl, xp)));
  float2 tail = fsub2(dl, fadd2(ep, es));
  tail = fadd2(tail, fsub2(fadd2(fadd2(na, nb), nc), lo));
  return fadd2(fsub2(dh, p), tail);
}
template <bool GEN>
R2_HD float2 res_interior(float2 dh, float2 dl, float2 xm, float2 x0, float2 xp, const Args& a) {
  return GEN ? res_pair_gen(dh, dl, xm, x0, xp, a) : res_pair(dh, dl, xm, x0, xp, a);
}
// The same for one row with double-word coefficients of any value (the
// special head and tail rows).
R2_HD float res_row(float dh, float dl, float xm, float x0, float xp, DWc ca, DWc cb, DWc cc) {
  float pa, pb, pc, ea, eb, ec;
  pa = mul_(ca.h, xm);
  ea = fma_(ca.h, xm, -pa);
  pb = mul_(cb.h, x0);
  eb = fma_(cb.h, x0, -pb);
  pc = mul_(cc.h, xp);
  ec = fma_(cc.h, xp, -pc);
  float s, es, p, ep;
  two_sum(pa, pc, s, es);
  two_sum(pb, s, p, ep);
  float tail = add_(dl, -add_(ep, es));
  tail = add_(tail, -add_(add_(ea, eb), ec));
  tail = add_(tail, -fma_(ca.l, xm, fma_(cb.l, x0, mul_(cc.l, xp))));
  return add_(add_(dh, -p), tail);
}

// s (x + d) for the FP32 solution x and its correction d (pairs) as two
// doubles: s_h x split exactly (its product error from an FMA), the small
// terms s_h d and s_l x added to that error, FastTwoSum, assembly.
R2_HD void out_pair(float2 x, float2 d, const Args& a, double& oa, double& ob) {
  float2 h, e;
  if (a.unit_scale) {
    two_sum2(x, d, h, e);
  } else {
    const float2 p = fmul2(a.sh, x);
    float2 u = ffma2(a.nsh, x, p);  // p - sh x = -(product error), exact
    u = ffma2(a.nsh, d, u);
    u = ffma2(a.nsl, x, u);         // u = -(error + sh d + sl x)
    h = fsub2(p, u);
    e = fsub2(fsub2(p, h), u);
  }
  oa = dw_to_f64(h.x, e.x);
  ob = dw_to_f64(h.y, e.y);
}
// s x without a correction (the FP32-only precision)
R2_HD void out_pair0(float2 x, const Args& a, double& oa, double& ob) {
  if (a.unit_scale) {
    oa = dw_to_f64(x.x, 0.f);
    ob = dw_to_f64(x.y, 0.f);
    return;
  }
  const float2 p = fmul2(a.sh, x);
  float2 u = ffma2(a.nsh, x, p);
  u = ffma2(a.nsl, x, u);
  const float2 h = fsub2(p, u);
  const float2 e = fsub2(fsub2(p, h), u);
  oa = dw_to_f64(h.x, e.x);
  ob = dw_to_f64(h.y, e.y);
}

// The compact scheme's one-sided boundary stencil (compact/rhs.py:21-31),
// in FP64, as a normalised double-word: sigma ((-5 r0 + 4 r1) + r2).
R2_HD void boundary_rhs(double r0, double r1, double r2, double sigma, float& h, float& l, unsigned& rmax) {
  const double v = dmul_(sigma, dadd_(dfma_(-5.0, r0, dmul_(4.0, r1)), r2));
  float hh, ll;
  split_f64(v, hh, ll, rmax);
  fast_two_sum(hh, ll, h, l);
}

}  // namespace r2
}  // namespace ntk
