// fixedsum.cuh — exact whole-cell sums in 128-bit fixed point.
//
// The three sums every time step needs (cs, xicat, xinaca over the cell's
// CRUs, cuda_Cell_Detailed.cu:435-456) are accumulated as value * 2^64 in
// two's-complement 128-bit integers.  FP32 values in the model's range
// (|v| < 2^40, magnitudes down to 2^-64) convert exactly, FP64 values are
// truncated below 2^-64; integer addition is exact and associative, so every
// CTA adds its tile's sum to the cell's accumulator with integer atomics in
// any order and the result is the same bits every run.  The cell update
// converts the total to FP64 with one rounding.  No FP64 arithmetic runs in
// the lattice CTAs, where it would cost the slow FP64 pipe.
#pragma once

#include <stdint.h>

namespace rh {

// Magnitudes at or above 2^kFxMaxExp are reported as invalid (the model's
// concentrations and currents are many orders below it).
constexpr int kFxMaxExp = 40;

__device__ __forceinline__ void fx_neg(uint64_t& lo, uint64_t& hi) {
  lo = ~lo + 1ull;
  hi = ~hi + (lo == 0ull ? 1ull : 0ull);
}

// v * 2^64 as (lo, hi), truncated toward zero; `bad` is set for non-finite
// values and |v| >= 2^kFxMaxExp (the result is then 0).
__device__ __forceinline__ void fx_from(float v, uint64_t& lo, uint64_t& hi, uint32_t& bad) {
  const uint32_t b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 0xffu);
  const uint64_t m = (uint64_t)((b & 0x7fffffu) | 0x800000u);  // 24 bits
  lo = 0ull;
  hi = 0ull;
  if (e >= 127 + kFxMaxExp) {  // also Inf and NaN (e = 255)
    bad = 1u;
    return;
  }
  if (e == 0) return;  // zero or subnormal: below 2^-126, under the resolution
  const int s = e - 86;  // v * 2^64 = m * 2^s, s < 81
  if (s >= 64) {
    hi = m << (s - 64);
  } else if (s >= 0) {
    lo = m << s;
    hi = s > 40 ? (m >> (64 - s)) : 0ull;
  } else if (s > -24) {
    lo = m >> (-s);
  }
  if (b >> 31) fx_neg(lo, hi);
}

__device__ __forceinline__ void fx_from(double v, uint64_t& lo, uint64_t& hi, uint32_t& bad) {
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ffull);
  const uint64_t m = (b & 0xfffffffffffffull) | 0x10000000000000ull;  // 53 bits
  lo = 0ull;
  hi = 0ull;
  if (e >= 1023 + kFxMaxExp) {
    bad = 1u;
    return;
  }
  if (e == 0) return;
  const int s = e - 1011;  // v * 2^64 = m * 2^s, s < 52
  if (s >= 0) {
    lo = m << s;
    hi = s > 11 ? (m >> (64 - s)) : 0ull;
  } else if (s > -53) {
    lo = m >> (-s);
  }
  if (b >> 63) fx_neg(lo, hi);
}

__device__ __forceinline__ void fx_add(uint64_t& lo, uint64_t& hi, uint64_t lo2, uint64_t hi2) {
  const uint64_t l = lo + lo2;
  hi = hi + hi2 + (l < lo ? 1ull : 0ull);
  lo = l;
}

// Warp sum; the total is valid in lane 0.
__device__ __forceinline__ void fx_warp_sum(uint64_t& lo, uint64_t& hi) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t l2 = __shfl_down_sync(0xffffffffu, lo, off);
    const uint64_t h2 = __shfl_down_sync(0xffffffffu, hi, off);
    fx_add(lo, hi, l2, h2);
  }
}

// Warp sum of one FP32 value per lane as value * 2^64 in 128-bit fixed
// point, the same in every lane.  Cheaper than fx_from + fx_warp_sum: the
// lanes align their 24-bit mantissas to the warp's largest exponent E
// (value = m * 2^(e - 150), m scaled by 2^(34 - (E - e)), so 32 of them stay
// below 2^63) and add them as 64-bit integers; only lanes
// more than 2^34 below the warp's largest value lose low bits (an error
// below 2^-58 of that value).  Integer adds, so the result does not depend
// on the order of the lanes; `bad` as in fx_from.
__device__ __forceinline__ void fx_warp_sum_f32(float v, uint64_t& lo, uint64_t& hi,
                                                uint32_t& bad) {
  const uint32_t b = __float_as_uint(v);
  uint32_t e = (b >> 23) & 0xffu;
  if (e >= 127u + kFxMaxExp) {  // also Inf and NaN; counted as 0
    bad = 1u;
    e = 0u;
  }
  const uint32_t E = __reduce_max_sync(0xffffffffu, e);
  const uint32_t m = e ? ((b & 0x7fffffu) | 0x800000u) : 0u;  // zero and subnormals: 0
  const int s = 34 - (int)(E - e);
  int64_t x = s >= 0 ? (int64_t)((uint64_t)m << s) : (s > -32 ? (int64_t)(m >> -s) : 0);
  if (b >> 31) x = -x;
  // The exact 64-bit sum over the warp as three 32-bit warp reductions:
  // x = xh 2^32 + xl with |xh| < 2^26 (|x| < 2^58), so the 32 high words
  // sum within a signed 32-bit integer, and the low words are summed in two
  // 16-bit halves (each sum below 2^21).
  {
    const int32_t xh = (int32_t)(x >> 32);
    const uint32_t xl = (uint32_t)x;
    const int32_t sh32 = __reduce_add_sync(0xffffffffu, xh);
    const uint32_t sa = __reduce_add_sync(0xffffffffu, xl & 0xffffu);
    const uint32_t sb = __reduce_add_sync(0xffffffffu, xl >> 16);
    x = (int64_t)((uint64_t)(int64_t)sh32 << 32) + ((int64_t)sb << 16) + (int64_t)sa;
  }
  // sum * 2^(E - 184) * 2^64 = x * 2^(E - 120), sh in [-120, 47]
  const int sh = (int)E - 120;
  const int64_t sx = x >> 63;  // sign fill
  if (sh >= 0) {
    lo = (uint64_t)x << sh;
    hi = sh ? (uint64_t)(x >> (64 - sh)) : (uint64_t)sx;
  } else {
    lo = -sh < 64 ? (uint64_t)(x >> -sh) : (uint64_t)sx;
    hi = (uint64_t)sx;
  }
}

// Adds (lo, hi) to the 128-bit accumulator acc[0..1] (lo word first).
__device__ __forceinline__ void fx_atomic_add(unsigned long long* acc, uint64_t lo, uint64_t hi) {
  const unsigned long long old = atomicAdd(acc, (unsigned long long)lo);
  const unsigned long long carry = (old + lo < old) ? 1ull : 0ull;
  atomicAdd(acc + 1, (unsigned long long)(hi + carry));
}

// The accumulated value as FP64 (one rounding).
__device__ __forceinline__ double fx_to_double(uint64_t lo, uint64_t hi) {
  const bool neg = (int64_t)hi < 0;
  if (neg) fx_neg(lo, hi);
  const double d = ((double)hi * 0x1.0p64 + (double)lo) * 0x1.0p-64;
  return neg ? -d : d;
}

}  // namespace rh
