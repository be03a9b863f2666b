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
// summation after Ogita, Rump and Oishi 2005), and a single DADD per row
// rebuilds the FP64 output.
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
// the rest rounded to a float (about 48 significant bits in all).  Valid for
// 2^-126 <= |x| < 2^128; zero maps to (0, 0); smaller magnitudes flush to
// zero; larger ones (and inf/nan) raise *range_flag.
__device__ __forceinline__ void split_f64(double x, float& hi, float& lo, unsigned& range_flag) {
  const unsigned h = (unsigned)__double2hiint(x);
  const unsigned l = (unsigned)__double2loint(x);
  const unsigned sign = h & 0x80000000u;
  const unsigned mag = h & 0x7fffffffu;
  const unsigned e = mag >> 20;  // biased double exponent
  // float bits of the truncated value: exponent re-biased by 1023-127=896
  const unsigned hb = __funnelshift_l(l, mag - (896u << 20), 3);
  // remaining 29 bits l[28:0] weigh 2^(e-1075); as a float: I2F then scale
  const float tail = __uint2float_rn(l & 0x1fffffffu);
  const float scale = __uint_as_float((e - 948u) << 23);  // 2^(e-1075), valid for e >= 949
  const bool normal = (e >= 897u) & (e <= 1150u);
  hi = normal ? __uint_as_float(hb | sign) : 0.0f;
  float t = __fmul_rn(tail, scale);
  t = (e >= 949u) ? t : 0.0f;
  lo = normal ? __uint_as_float(__float_as_uint(t) | sign) : 0.0f;
  range_flag |= (e > 1150u) ? 1u : 0u;
}

// float -> double by bit manipulation (normal floats and zero; denormals
// flush to zero).
__device__ __forceinline__ double f32_to_f64_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned m = b & 0x7fffffffu;
  unsigned hi = (m >> 3) + (896u << 20);
  hi = (m >= 0x00800000u) ? hi : 0u;
  const unsigned lo = (m >= 0x00800000u) ? (b << 29) : 0u;
  return __hiloint2double((int)(hi | (b & 0x80000000u)), (int)lo);
}

// hi + lo (a normalised double-word) rounded to the nearest double
__device__ __forceinline__ double dw_to_f64(float hi, float lo) {
#ifdef NTK_F2D_HW
  return (double)hi + (double)lo;
#else
  return f32_to_f64_bits(hi) + f32_to_f64_bits(lo);
#endif
}

// ---------------------------------------------------------------------------
// small utilities
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

}  // namespace ntk
