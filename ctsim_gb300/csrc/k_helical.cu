// k_helical.cu -- helical 180-degree linear interpolation and half-scan
// feathering on sm_103a (Projections::Helical180LI_Equiangular and
// Projections::HalfScanFeather, libctsim/projections.cpp:231-439).
//
// The reference scatters every input ray into the output view set with FP64
// weights and accumulates in FP32 in view order.  Each output sample receives
// at most two rays: its own (views before pi+fan) and its complementary ray
// (detector mirrored, view shifted by 2*gamma - pi).  The kernels here gather
// instead of scatter: one thread per output sample finds both source rays,
// evaluates the same FP64 region tests and weights, and adds them in the
// reference's order with the reference's FP32 rounding, so the result is
// bit-identical and deterministic.
//
// Equilinear restatement (no reference counterpart; the reference refuses
// that geometry, projections.cpp:214-218): the same algorithm with each
// detector's true fan angle gamma = atan(pos / SDL), pos its distance from
// the integer detector centre (projections.cpp:1366-1370 maps the equilinear
// detector to fan angles the same way).
#include "ctgpu_internal.h"
#include "k_fpconv.cuh"

namespace ctgpu {

namespace {

__device__ __forceinline__ int nearest_int(double x) { return x > 0 ? (int)(x + 0.5) : (int)(x - 0.5); }

// fan angle of detector id (projections.cpp:247: integer centre (nDet-1)/2)
__device__ __forceinline__ double det_gamma(const HelicalLaunch& L, int id) {
  const double pos = (id - (L.nDet - 1) / 2) * L.dgamma;
  return L.equilinear ? atan(pos / L.sdl) : pos;
}

// weight of input ray (iv, id) in the 180LI sum; false outside regions 2-7
// (projections.cpp:306-350)
__device__ bool li_weight(double beta, double gamma, double fan, double* w) {
  const double PI = kPi;
  if (!((beta > fan - 2 * gamma) && (beta < 2 * PI + fan - 2 * gamma))) return false;
  if (beta > fan - 2 * gamma && beta <= 2 * fan) *w = (beta + 2 * gamma - fan) / (PI + 2 * gamma);
  else if (beta > 2 * fan && beta <= PI - 2 * gamma) *w = (beta + 2 * gamma - fan) / (PI + 2 * gamma);
  else if (beta > PI - 2 * gamma && beta <= PI + fan) *w = (beta + 2 * gamma - fan) / (PI + 2 * gamma);
  else if (beta > PI + fan && beta <= PI + 2 * fan - 2 * gamma) *w = (2 * PI - beta - 2 * gamma + fan) / (PI - 2 * gamma);
  else if (beta > PI + 2 * fan - 2 * gamma && beta <= 2 * PI) *w = (2 * PI - beta - 2 * gamma + fan) / (PI - 2 * gamma);
  else if (beta > 2 * PI && beta <= 2 * PI + fan - 2 * gamma) *w = (2 * PI - beta - 2 * gamma + fan) / (PI - 2 * gamma);
  else return false;
  return true;
}

}  // namespace

__global__ void helical180li_kernel(HelicalLaunch L) {
  const int vo = blockIdx.x;                  // output view
  const int nDet = L.nDet;
  const double dbeta = L.dbeta, fan = L.fan, PI = kPi;
  const int last = L.nViewOut - 1, lastAcq = 2 * last;
  for (int dO = threadIdx.x; dO < nDet; dO += blockDim.x) {
    float o = 0.f;
    // own ray: iv = vo, id = dO, valid while beta < pi + fan
    {
      int iv = vo, id = dO;
      double beta = iv * dbeta;
      double gamma = det_gamma(L, id);
      double w;
      if (beta < PI + fan && li_weight(beta, gamma, fan, &w))
        o = (float)((double)o + w * (double)L.in[(size_t)(iv + L.offsetView) * L.pitch + id]);
    }
    // complementary ray: id = nDet-1-dO, nearest(iv + (2 gamma - pi)/dbeta) == vo
    {
      int id = nDet - 1 - dO;
      double gamma = det_gamma(L, id);
      int guess = (int)floor(vo - (2 * gamma - PI) / dbeta);
      for (int iv = guess - 2; iv <= guess + 2; iv++) {
        if (iv < 0 || iv > lastAcq) continue;
        double beta = iv * dbeta;
        if (beta < PI + fan) continue;
        int nv = nearest_int(((iv * dbeta) + 2 * gamma - PI) / dbeta);
        if (nv != vo) continue;
        double w;
        if (li_weight(beta, gamma, fan, &w))
          o = (float)((double)o + w * (double)L.in[(size_t)(iv + L.offsetView) * L.pitch + id]);
      }
    }
    L.out[(size_t)vo * L.pitch + dO] = o;
  }
}

// feather weight w1 of the complementary sample at (beta1, gamma1)
// (projections.cpp:408-421); false for the reference's "Shouldn't be here" case
__device__ bool feather_w1(double beta1, double gamma1, double fan, double* w1) {
  const double PI = kPi;
  double x;
  if (beta1 <= (fan - 2 * gamma1)) x = beta1 / (fan - 2 * gamma1);
  else if ((fan - 2 * gamma1 <= beta1) && beta1 <= PI - 2 * gamma1) x = 1;
  else if ((PI - 2 * gamma1 <= beta1) && (beta1 <= PI + fan)) x = (PI + fan - beta1) / (fan + 2 * gamma1);
  else return false;
  *w1 = (3 * x - 2 * x * x) * x;
  return true;
}

__global__ void halfscan_feather_kernel(HelicalLaunch L) {
  const int v = blockIdx.x;
  const int nDet = L.nDet, nView = L.nViewOut;
  const double dbeta = L.dbeta, fan = L.fan, PI = kPi;
  const double sf = nView * L.dbeta / PI;
  for (int d = threadIdx.x; d < nDet; d += blockDim.x) {
    float x = L.in[(size_t)v * L.pitch + d];
    double beta = v * dbeta;
    double gamma = det_gamma(L, d);
    if (beta >= PI - 2 * gamma) {
      // redundant sample: keeps weight w2 = 1 - w1 of its complement
      int iv1 = nearest_int(((v * dbeta) + 2 * gamma - PI) / dbeta);
      double w1;
      if (!feather_w1(iv1 * dbeta, -gamma, fan, &w1)) { atomicOr(L.status, kStatusFeatherRange); w1 = 0; }
      x = (float)((double)x * (1 - w1));
    } else {
      // complement target of the redundant sample (iv2, nDet-1-d), if any
      int id2 = nDet - 1 - d;
      double gamma2 = det_gamma(L, id2);
      int guess = (int)floor(v + (PI - 2 * gamma2) / dbeta);
      for (int iv2 = guess - 2; iv2 <= guess + 2; iv2++) {
        if (iv2 < 0 || iv2 >= nView) continue;
        double beta2 = iv2 * dbeta;
        if (!(beta2 >= PI - 2 * gamma2)) continue;
        int iv1 = nearest_int(((iv2 * dbeta) + 2 * gamma2 - PI) / dbeta);
        if (iv1 != v) continue;
        double w1;
        if (!feather_w1(v * dbeta, -gamma2, fan, &w1)) { atomicOr(L.status, kStatusFeatherRange); w1 = 0; }
        float x2 = L.in[(size_t)iv2 * L.pitch + id2];
        x = (float)((double)x2 * w1);
      }
    }
    L.out[(size_t)v * L.pitch + d] = (float)((double)x * sf);
  }
}

cudaError_t launch_helical180li(const HelicalLaunch& L, cudaStream_t s) {
  helical180li_kernel<<<L.nViewOut, 128, 0, s>>>(L);
  return cudaGetLastError();
}
cudaError_t launch_halfscan_feather(const HelicalLaunch& L, cudaStream_t s) {
  halfscan_feather_kernel<<<L.nViewOut, 128, 0, s>>>(L);
  return cudaGetLastError();
}

}  // namespace ctgpu

// ---------------------------------------------------------------------------
// Many slices of one helical data set.  The 180LI weights and complementary
// rays of an output sample, and the feathering that follows, depend only on
// the geometry -- not on the interpolation view -- so they are tabulated once
// (same FP64 expressions as the kernels above) and every run gathers all
// slices in one launch: out = sf * (w_f * interp(vs, ds)) with
// interp = own-ray term then complementary-ray term, in the reference's order
// and FP32 roundings.
// ---------------------------------------------------------------------------
namespace ctgpu {

__global__ void helical_tables_kernel(HelicalLaunch L, const double* __restrict__ gammaTab,
                                      HelicalTap* __restrict__ interp,
                                      FeatherTap* __restrict__ feather) {
  const int vo = blockIdx.x;
  const int nDet = L.nDet;
  const double dbeta = L.dbeta, fan = L.fan, PI = kPi;
  const int last = L.nViewOut - 1, lastAcq = 2 * last;
  for (int dO = threadIdx.x; dO < nDet; dO += blockDim.x) {
    HelicalTap t;
    t.w0 = 0.0;
    t.wc = 0.0;
    t.own = 0;
    t.ivc = -1;
    {
      double beta = vo * dbeta, gamma = gammaTab[dO], w;
      if (beta < PI + fan && li_weight(beta, gamma, fan, &w)) {
        t.own = 1;
        t.w0 = w;
      }
    }
    {
      int id = nDet - 1 - dO;
      double gamma = gammaTab[id];
      int guess = (int)floor(vo - (2 * gamma - PI) / dbeta);
      for (int iv = guess - 2; iv <= guess + 2; iv++) {
        if (iv < 0 || iv > lastAcq) continue;
        double beta = iv * dbeta;
        if (beta < PI + fan) continue;
        int nv = nearest_int(((iv * dbeta) + 2 * gamma - PI) / dbeta);
        if (nv != vo) continue;
        double w;
        if (li_weight(beta, gamma, fan, &w)) {
          t.ivc = iv;
          t.wc = w;
        }
      }
    }
    interp[(size_t)vo * nDet + dO] = t;
    if (feather) {
      // halfscan_feather_kernel's choice for output sample (vo, dO)
      FeatherTap f;
      f.v = vo;
      f.d = dO;
      f.w = 1.0;
      f.bad = 0;
      double beta = vo * dbeta, gamma = gammaTab[dO];
      if (beta >= PI - 2 * gamma) {
        int iv1 = nearest_int(((vo * dbeta) + 2 * gamma - PI) / dbeta);
        double w1;
        if (!feather_w1(iv1 * dbeta, -gamma, fan, &w1)) { f.bad = 1; w1 = 0; }
        f.w = 1 - w1;
      } else {
        int id2 = nDet - 1 - dO;
        double gamma2 = gammaTab[id2];
        int guess = (int)floor(vo + (PI - 2 * gamma2) / dbeta);
        for (int iv2 = guess - 2; iv2 <= guess + 2; iv2++) {
          if (iv2 < 0 || iv2 > last) continue;
          double beta2 = iv2 * dbeta;
          if (!(beta2 >= PI - 2 * gamma2)) continue;
          int iv1 = nearest_int(((iv2 * dbeta) + 2 * gamma2 - PI) / dbeta);
          if (iv1 != vo) continue;
          double w1;
          if (!feather_w1(vo * dbeta, -gamma2, fan, &w1)) { f.bad = 1; w1 = 0; }
          f.v = iv2;
          f.d = id2;
          f.w = w1;
        }
      }
      feather[(size_t)vo * nDet + dO] = f;
    }
  }
}

// 180LI value of output sample (vo, d) of the slice whose first input view
// is off: the reference's o = (float)((double)o + w * (double)in) per ray, o
// starting at 0.f, with the conversions on the integer pipe (k_fpconv.cuh).
// FP64 is the binding pipe of this kernel: 64 slices of 769 x 1024 took
// 1.37 ms with the hardware conversions, 1.18 ms without, the FP64 pipe
// still 87 % busy with the multiplications and the addition
__device__ __forceinline__ float helical_interp(const HelicalTap& t, const float* in, int off,
                                                int pitch, int nDet, int vo, int d) {
  float o = 0.f;
  if (t.own)   // (double)0.f + p
    o = f64_to_f32_rn(plus_zero(t.w0 * f32_to_f64(in[(size_t)(vo + off) * pitch + d])));
  if (t.ivc >= 0)
    o = f64_to_f32_rn(f32_to_f64(o) +
                      t.wc * f32_to_f64(in[(size_t)(t.ivc + off) * pitch + (nDet - 1 - d)]));
  return o;
}

// grid (output views, slices)
__global__ void helical_slices_kernel(HelicalSlicesLaunch L) {
  const int vo = blockIdx.x, z = blockIdx.y;
  const int off = L.offsets[z];
  float* out = L.out + (size_t)z * L.outSliceStride + (size_t)vo * L.outPitch;
  for (int d = threadIdx.x; d < L.nDet; d += blockDim.x) {
    float x;
    if (L.feather) {
      const FeatherTap f = L.feather[(size_t)vo * L.nDet + d];
      if (f.bad) atomicOr(L.status, kStatusFeatherRange);
      x = helical_interp(L.interp[(size_t)f.v * L.nDet + f.d], L.in, off, L.inPitch, L.nDet, f.v,
                         f.d);
      x = f64_to_f32_rn(f32_to_f64(x) * f.w);
      x = f64_to_f32_rn(f32_to_f64(x) * L.sf);
    } else {
      x = helical_interp(L.interp[(size_t)vo * L.nDet + d], L.in, off, L.inPitch, L.nDet, vo, d);
    }
    out[d] = x;
  }
}

cudaError_t launch_helical_tables(const HelicalLaunch& L, const double* gammaTab,
                                  HelicalTap* interp, FeatherTap* feather, cudaStream_t s) {
  helical_tables_kernel<<<L.nViewOut, 128, 0, s>>>(L, gammaTab, interp, feather);
  return cudaGetLastError();
}

cudaError_t launch_helical_slices(const HelicalSlicesLaunch& L, cudaStream_t s) {
  if (L.nSlices <= 0) return cudaSuccess;
  if (L.nSlices > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid(L.nViewOut, L.nSlices);
  helical_slices_kernel<<<grid, 128, 0, s>>>(L);
  return cudaGetLastError();
}

}  // namespace ctgpu
