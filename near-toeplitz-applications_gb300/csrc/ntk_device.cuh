// ntk_device.cuh -- device helpers shared by the ntk kernels (sm_103a).
//
// Double-word ("float-float") arithmetic for the FP32 + refinement path.
// On GB300 the FP64 pipe issues about 1.7 operations per clock per SM
// (measured: DFMA and DADD at ~500 G instr/s over 152 SMs, 64-cycle
// latency) against 128 FP32 operations, and the double->float conversion
// runs at the same slow rate.  The refinement path therefore keeps FP64
// out of its inner loops: FP64 inputs are split into two floats with
// integer operations, the residual is formed with error-free
// transformations (TwoSum / TwoProd, Knuth 1969, Dekker 1971; accurate
// summation after Ogita, Rump and Oishi 2005), and the FP64 output is
// assembled from the double-word with integer operations.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ntk {

// ---------------------------------------------------------------------------
// error-free transformations (rounding to nearest, no contraction)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// ---------------------------------------------------------------------------
// FP64 <-> double-word without the FP64 pipe
// ---------------------------------------------------------------------------
// Splits x into hi + lo with hi = x truncated to 24 significant bits and lo
// the next 23 bits (47 significant bits in all), using only INT and FP32
// operations: the double->float conversion and I2F both issue on GB300's slow
// FP64-rate pipe.  lo is built exactly with the magic-number trick: the 23
// bits are placed under the exponent of 2^23 and 2^23 is subtracted.
// Valid for 2^-80 <= |x| < 2^128 (lo is dropped below 2^-80, hi and lo are 0
// below 2^-126); larger magnitudes, inf and nan raise range_flag.
__device__ __forceinline__ void split_f64(double x, float& hi, float& lo, unsigned& range_flag) {
  const unsigned h = (unsigned)__double2hiint(x);
  const unsigned l = (unsigned)__double2loint(x);
  const unsigned mag = h & 0x7fffffffu;
  // ((h - 896<<20) << 3) | (l >> 29): the sign bit is shifted out
  const unsigned hb = __funnelshift_l(l, h - (896u << 20), 3);
  const unsigned sign = h & 0x80000000u;
  const float hv = __uint_as_float((hb & 0x7fffffffu) | sign);
  // bits l[28:6] as an exact float integer, weight 2^(e-1069)
  const float t = __fsub_rn(__uint_as_float(((l >> 6) & 0x007fffffu) | 0x4b000000u), 8388608.0f);
  const float sc = __uint_as_float((hb & 0x7f800000u) - (46u << 23));
  const float lv = __uint_as_float(__float_as_uint(__fmul_rn(t, sc)) | sign);
  hi = (mag >= (897u << 20)) ? hv : 0.0f;
  lo = (mag >= (943u << 20)) ? lv : 0.0f;
  range_flag |= (mag >= (1151u << 20)) ? 1u : 0u;
}

// hi + lo (a normalised double-word: |lo| <= ulp(hi)/2) as a double, with
// INT and FP32 operations only (no DADD on the slow FP64 pipe).  lo is
// expressed in units of 64 ulps of hi-as-a-double: lo * 2^(46 - e_hi) lies
// within +-2^22, so adding 1.5 * 2^23 rounds it to an integer k held in the
// float's low mantissa bits, and k * 64 is added to the 64-bit pattern of
// hi.  hi's low 29 mantissa bits are zero and |64 k| <= 2^28, so the sum
// never crosses a binade, except below an exact power of two (hi = +-2^e
// and lo of the other sign), where the double's ulp halves and k is doubled.
// Relative error <= 2^-47, the precision the double-word carries; |hi| below
// 2^-81 (and zero) gives zero.
__device__ __forceinline__ double dw_to_f64(float hi, float lo) {
  const unsigned bh = __float_as_uint(hi);
  const unsigned eh = bh & 0x7f800000u;
  // 2^(46 - e_hi) carrying hi's sign: k > 0 moves away from zero
  const float sc = __uint_as_float(((300u << 23) - eh) | (bh & 0x80000000u));
  const float t = __fmaf_rn(lo, sc, 12582912.0f);  // one rounding: k = round(lo * sc)
  int k = (int)(__float_as_uint(t) - 0x4b400000u);
  if ((bh & 0x007fffffu) == 0u && k < 0) k *= 2;
  const unsigned dhi = ((bh & 0x7fffffffu) >> 3) + (896u << 20);
  const unsigned dlo = bh << 29;
  unsigned long long bits = (((unsigned long long)dhi << 32) | dlo) + (unsigned long long)((long long)k << 6);
  bits = (eh >= (46u << 23)) ? bits : 0ull;
  return __longlong_as_double((long long)(bits | ((unsigned long long)(bh & 0x80000000u) << 32)));
}

// ---------------------------------------------------------------------------
// asynchronous global -> shared copies (cp.async, 8 bytes).  src_bytes = 0
// zero-fills the destination without reading src.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, unsigned src_bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// border rows of the batch windows (ntk_batch.cu, ntk_batch_refine.cu)
// ---------------------------------------------------------------------------
// Border rows of windows g = first .. first + count - 1 copied from work into
// d by one warp (geom(g, base, lo, blo, bhi, hi): rows base + [lo, blo) and
// base + [bhi, hi)).  Segments are short (a few dozen rows), so the warp
// loads four windows' first 64 rows of each segment before storing any:
// 16 loads in flight per lane instead of a chain of round trips.
template <class GEOM>
__device__ __forceinline__ void border_copy(const double* work, double* d, int first, int count, unsigned lane,
                                            GEOM geom) {
  for (int g0 = first; g0 < first + count; g0 += 4) {
    double v[4][4];
    long long at[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      long long base = 0;
      int lo = 0, blo = 0, bhi = 0, hi = 0;
      if (g0 + i < first + count) geom(g0 + i, base, lo, blo, bhi, hi);
      const int r[4] = {lo + (int)lane, lo + 32 + (int)lane, bhi + (int)lane, bhi + 32 + (int)lane};
      const int e[4] = {blo, blo, hi, hi};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        at[i][q] = r[q] < e[q] ? base + r[q] : -1;
        v[i][q] = at[i][q] >= 0 ? __ldcg(work + at[i][q]) : 0.0;
      }
      // rows beyond 64 of a segment (long halos): plain loop
      for (int rr = lo + 64 + (int)lane; rr < blo; rr += 32) d[base + rr] = __ldcg(work + base + rr);
      for (int rr = bhi + 64 + (int)lane; rr < hi; rr += 32) d[base + rr] = __ldcg(work + base + rr);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (at[i][q] >= 0) d[at[i][q]] = v[i][q];
  }
}

// The nt threads of a CTA copy a system's border rows (absolute row indices
// in rows[0, count), ntk_batch_borders.h) from work into d, eight rows a
// thread in flight.
__device__ __forceinline__ void row_copy(const double* work, double* d, const long long* __restrict__ rows,
                                         int count, int t, int nt) {
  for (int base = 0; base < count; base += 8 * nt) {
    long long at[8];
    double v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int i = base + t + q * nt;
      at[q] = i < count ? __ldg(rows + i) : -1;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = at[q] >= 0 ? __ldcg(work + at[q]) : 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (at[q] >= 0) d[at[q]] = v[q];
  }
}

// ---------------------------------------------------------------------------
// small utilities
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

}  // namespace ntk
