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
// asynchronous global -> shared copies (cp.async, 8 bytes).  src_bytes = 0
// zero-fills the destination without reading src.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, unsigned src_bytes) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// ---------------------------------------------------------------------------
// small utilities
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

}  // namespace ntk
