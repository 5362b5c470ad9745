// k_fpconv.cuh -- FP32 <-> FP64 conversions by integer operations, for the
// kernels that reproduce FP64 expressions of the reference bit for bit
// (k_helical.cu).  On this GPU the conversions run on the FP64 pipe, 1/64 of
// the FP32 rate; these forms use the integer pipe instead, and fall back to
// the hardware conversion for the rare inputs they do not cover.
//
//   f32_to_f64(f):     exact (every float is a double); by fields for normal
//                      floats and zeros
//   f64_to_f32_rn(d):  IEEE 754 round to nearest, ties to even; by fields
//                      where the result is a normal float or overflows to
//                      infinity by rounding
//   plus_zero(d):      d + 0.0 (turns -0.0 into +0.0, leaves the rest)
//
// Host and device: tests/cpp/fpconv_check.cpp compares them with the CPU's
// own conversions.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define CTGPU_FPC __host__ __device__ __forceinline__
#else
#define CTGPU_FPC inline
#endif

namespace ctgpu {

CTGPU_FPC uint64_t fpc_bits64(double d) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t u;
  memcpy(&u, &d, sizeof u);
  return u;
#endif
}
CTGPU_FPC double fpc_double(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double d;
  memcpy(&d, &u, sizeof d);
  return d;
#endif
}
CTGPU_FPC uint32_t fpc_bits32(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, sizeof u);
  return u;
#endif
}
CTGPU_FPC float fpc_float(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, sizeof f);
  return f;
#endif
}

CTGPU_FPC double f32_to_f64(float f) {
  const uint32_t u = fpc_bits32(f);
  const uint32_t e = (u >> 23) & 0xFFu;   // biased exponent
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  if (e == 0u || e == 255u) {
    if ((u & 0x7FFFFFFFu) == 0u) return fpc_double(sign);   // +-0
    return (double)f;                                       // subnormal, inf, nan
  }
  // exponent bias 127 -> 1023, 23-bit fraction -> the top of the 52-bit one
  return fpc_double(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7FFFFFu) << 29));
}

CTGPU_FPC float f64_to_f32_rn(double d) {
  const uint64_t u = fpc_bits64(d);
  const int e = (int)((u >> 52) & 0x7FFu) - 896;   // the float's biased exponent
  if (e <= 0 || e >= 255) return (float)d;          // zero, subnormal, out of range, inf, nan
  const uint64_t frac = u & 0xFFFFFFFFFFFFFull;     // 52 bits
  const uint32_t m = (uint32_t)(frac >> 29);        // the float's 23
  const uint32_t rest = (uint32_t)(frac & 0x1FFFFFFFull);   // the 29 dropped
  uint32_t b = ((uint32_t)(u >> 32) & 0x80000000u) | ((uint32_t)e << 23) | m;
  // round half to even; a carry out of the fraction raises the exponent
  // (and past the largest finite float gives infinity, as the rounding must)
  if (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) b += 1u;
  return fpc_float(b);
}

CTGPU_FPC double plus_zero(double d) {
  return (fpc_bits64(d) << 1) == 0 ? 0.0 : d;   // +-0 -> +0
}

}  // namespace ctgpu
