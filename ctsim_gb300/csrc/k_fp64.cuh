// k_fp64.cuh -- FP64 helpers for the set-up kernels (k_raysum.cu,
// k_backproject.cu).  FP64 runs at 1/64 of the FP32 rate on this GPU, and the
// library's correctly rounded 1/sqrt, division and atan take tens of FP64
// instructions each; these take a few, to about 1e-13 relative (reciprocals)
// and 2e-15 absolute (arctangent), far below the FP32 values they feed.
#pragma once

#include <array>
#include <cmath>

#include "ctgpu_internal.h"

namespace ctgpu {

// FP64 1/sqrt(x) (x > 0) and 1/x (|x| in [1e-300, 1e300]): the hardware's
// approximate FP64 estimate (PTX rsqrt.approx.f64 / rcp.approx.f64, about
// 2^-22 relative) and one Newton-Raphson step.
__device__ __forceinline__ double rsqrt_nr(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  return y * fma(-0.5 * x * y, y, 1.5);
}
__device__ __forceinline__ double rcp_nr(double x) {
  if (!(fabs(x) > 1e-300 && fabs(x) < 1e300)) return 1.0 / x;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  return fma(y, fma(-x, y, 1.0), y);
}

// atan(j / 64), j = 0..64, by the host's FP64 atan; passed to kernels by value
struct Atan64 {
  double v[65];
};
inline const Atan64& atan64_table() {
  static const Atan64 tab = [] {
    Atan64 t{};
    for (int j = 0; j <= 64; j++) t.v[j] = std::atan(j / 64.0);
    return t;
  }();
  return tab;
}

// atan2(s, c) in FP64 for c >= |s| (angles within pi/4 of the +x axis) by the
// table-driven method: with z = |s|/c and j the nearest of 64 z,
// atan z = atan(j/64) + atan r, r = (z - j/64) / (1 + z j/64), |r| <= 1/128
// (to within the FP32 choice of j), and atan r by its Taylor series to r^7
// (truncation below 2e-20).  Other arguments take the library's atan2.
__device__ __forceinline__ double atan2_tab(double s, double c, const double* tab) {
  const double as = fabs(s);
  if (!(c > 0.0 && as <= c && c < 1e30)) return atan2(s, c);
  int j = __float2int_rn(64.f * __fdividef((float)as, (float)c));
  j = min(max(j, 0), 64);
  const double tj = j * (1.0 / 64.0);
  const double r = fma(-c, tj, as) * rcp_nr(fma(as, tj, c));
  const double r2 = r * r;
  const double p = fma(fma(r2, -1.0 / 7.0, 1.0 / 5.0), r2, -1.0 / 3.0);
  const double a = tab[j] + fma(p * r2, r, r);
  return s < 0.0 ? -a : a;
}

}  // namespace ctgpu
