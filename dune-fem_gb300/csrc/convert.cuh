// float <-> double conversions in integer arithmetic, from the IEEE 754
// binary32 / binary64 formats.  On this GPU a hardware conversion between
// the two runs on the FP64 pipe, which is ~60 times narrower than the FP32
// pipe; elementwise kernels that convert every element would be bound by it.
// These give the same results as the hardware's round-to-nearest-even
// conversions for every input (normal, subnormal, zero, infinity; NaN stays
// a NaN); gbfem_selftest_conversions checks that on the device.
#pragma once
#include <cstdint>

namespace gbfem {

// binary64 -> binary32, round to nearest, ties to even
__device__ __forceinline__ float f64_to_f32_rn(double d) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
  const uint32_t sign = uint32_t(b >> 32) & 0x80000000u;
  const int e = int((b >> 52) & 0x7FF);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (m ? 0x00400000u : 0u));
  int fe = e - 1023 + 127;  // binary32 biased exponent
  if (fe >= 0xFF) return __uint_as_float(sign | 0x7F800000u);
  unsigned long long full;
  int shift;
  if (fe >= 1) {  // normal result: drop 29 of the 52 fraction bits
    full = m;
    shift = 29;
  } else {  // subnormal result (or zero): the implicit bit joins the fraction
    if (e == 0) return __uint_as_float(sign);  // |d| < 2^-1022
    shift = 30 - fe;
    if (shift > 53) return __uint_as_float(sign);  // below half the smallest subnormal
    full = m | (1ull << 52);
    fe = 0;
  }
  const unsigned long long kept = full >> shift;
  const unsigned long long rem = full & ((1ull << shift) - 1);
  const unsigned long long half = 1ull << (shift - 1);
  uint32_t r = sign | (uint32_t(fe) << 23) | uint32_t(kept);
  if (rem > half || (rem == half && (kept & 1ull))) r += 1u;  // a carry moves into the exponent correctly
  return __uint_as_float(r);
}

// binary32 -> binary64 (exact)
__device__ __forceinline__ double f32_to_f64(float f) {
  const uint32_t b = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
  const uint32_t e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
  unsigned long long r;
  if (e == 0xFFu) {
    r = sign | (0x7FFull << 52) | ((unsigned long long)m << 29);
  } else if (e != 0u) {
    r = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
  } else if (m == 0u) {
    r = sign;
  } else {  // subnormal: m 2^-149 with the leading bit at position k
    const int k = 31 - __clz(m);
    r = sign | ((unsigned long long)(k - 149 + 1023) << 52) | (((unsigned long long)m << (52 - k)) & 0xFFFFFFFFFFFFFull);
  }
  return __longlong_as_double(static_cast<long long>(r));
}

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(double v) { return f64_to_f32_rn(v); }
template <typename T> __device__ __forceinline__ T from_f32(float v);
template <> __device__ __forceinline__ float from_f32<float>(float v) { return v; }
template <> __device__ __forceinline__ double from_f32<double>(float v) { return f32_to_f64(v); }

}  // namespace gbfem
