// k_rows.cuh -- interval rows of filtered views for the table-family
// backprojection: one element per detector interval [g, g+1) holding the
// coefficients of the interpolant on it, in powers of the fraction t.
//   nearest: the sample f[g]
//   linear:  (f[g], f[g+1] - f[g])
//   cubic:   the CubicPolyInterpolator's Lagrange polynomial through
//            f[g-1..g+2] (libctsupport/interpolator.cpp:37-75), its first and
//            last intervals linear
// and zero outside the detector (the reference's value there).  Shared by
// interval_rows_kernel (k_backproject.cu) and the filter kernel that writes
// the rows from its own output (k_filter.cu), so both give the same bits.
#pragma once

#include "ctgpu_internal.h"

namespace ctgpu {

template <int INTERP> struct RowElem { typedef float T; };
template <> struct RowElem<kLinear> { typedef float2 T; };
template <> struct RowElem<kCubic> { typedef float4 T; };

// element of interval g of a row of n samples; f(i) reads sample i (called
// for 0 <= i < n only)
template <int INTERP, typename F>
__device__ __forceinline__ typename RowElem<INTERP>::T interval_elem(const F& f, int g, int n) {
  if constexpr (INTERP == kNearest) {
    return (g >= 0 && g < n) ? f(g) : 0.f;
  } else if constexpr (INTERP == kLinear) {
    float2 e = make_float2(0.f, 0.f);
    if (g >= 0 && g <= n - 2) {
      const float f0 = f(g);
      e = make_float2(f0, f(g + 1) - f0);
    }
    return e;
  } else {
    float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
    if (g == 0 || g == n - 2) {
      const float f0 = f(g);
      e.x = f0;
      e.y = f(g + 1) - f0;
    } else if (g >= 1 && g <= n - 3) {
      const float fm = f(g - 1), f0 = f(g), f1 = f(g + 1), f2 = f(g + 2);
      e.x = f0;
      e.y = fmaf(-1.f / 6.f, f2, fmaf(-1.f / 3.f, fm, fmaf(-0.5f, f0, f1)));
      e.z = fmaf(0.5f, fm + f1, -f0);
      e.w = fmaf(1.f / 6.f, f2 - fm, 0.5f * (f0 - f1));
    }
    return e;
  }
}

}  // namespace ctgpu
