// k_rebin.cu -- fan-beam to parallel rebinning on sm_103a
// (Projections::interpolateToParallel, libctsim/projections.cpp:1250-1328,
// with ParallelRaysums :1339-1469 and LinearInterpolator,
// include/interpolator.h:187-266).
//
// Every fan-beam sample (view v, detector d) is the parallel ray at angle
// theta = normalize(viewAngle_v + gamma_d) and signed distance
// t = FL sin(gamma_d).  All samples of one detector share t, so the reference's
// sort by (t, theta) groups them per detector (the host orders the detectors
// by t) and sorts each group by theta.  Pass 1 (one CTA per detector): the
// group's (theta, raysum) pairs are sorted in shared memory by a bitonic
// network (ties by view index) and linearly interpolated at the output view
// angles -> an intermediate [view][group] FP32 array, as the reference stores
// it.  Pass 2 (one CTA per output view): the row is interpolated from the
// groups' t positions to the output detector positions.  FP64 arithmetic
// as the reference, FP32 storage between and after.
#include "ctgpu_internal.h"

namespace ctgpu {

namespace {

constexpr double kTwoPiRb = 6.28318530717958647692;

__device__ __forceinline__ double normalize_angle(double th) {   // mathfuncs.cpp:72-81
  while (th < 0.) th += kTwoPiRb;
  while (th >= kTwoPiRb) th -= kTwoPiRb;
  return th;
}

// LinearInterpolator::interpolate (interpolator.h:203-265), x ascending, values
// outside the range clamp to the end samples
template <class Y>
__device__ double lin_interp(const double* x, const Y* y, int n, double dX) {
  int iLower = -1, iUpper = n;
  while (iUpper - iLower > 1) {
    int iMiddle = (iUpper + iLower) >> 1;
    if (dX >= x[iMiddle]) iLower = iMiddle;
    else iUpper = iMiddle;
  }
  if (dX == x[0] || dX < x[0]) return (double)y[0];
  if (dX == x[n - 1] || dX > x[n - 1]) return (double)y[n - 1];
  if (iLower < 0 || iLower >= n) return 0.0;
  const double y0 = (double)y[iLower], y1 = (double)y[iUpper];
  return y0 + (y1 - y0) * ((dX - x[iLower]) / (x[iUpper] - x[iLower]));
}

}  // namespace

__global__ void __launch_bounds__(256) rebin_theta_kernel(RebinLaunch L) {
  extern __shared__ __align__(16) unsigned char smr[];
  const int n = L.sortN;
  double* key = reinterpret_cast<double*>(smr);
  float* val = reinterpret_cast<float*>(key + n);
  int* idx = reinterpret_cast<int*>(val + n);
  const int d = blockIdx.x;
  const double gam = L.gam[d];
  for (int v = threadIdx.x; v < n; v += blockDim.x) {
    if (v < L.nView) {
      key[v] = normalize_angle(L.angles[v] + gam);
      val[v] = L.in[(size_t)v * L.pitch + d];
    } else {
      key[v] = __longlong_as_double(0x7ff0000000000000LL);   // +inf: padding sorts last
      val[v] = 0.f;
    }
    idx[v] = v;
  }
  __syncthreads();
  // bitonic sort ascending by (key, idx)
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const bool up = (i & k) == 0;
          const bool gt = key[i] > key[p] || (key[i] == key[p] && idx[i] > idx[p]);
          if (gt == up) {
            double tk = key[i]; key[i] = key[p]; key[p] = tk;
            float tv = val[i]; val[i] = val[p]; val[p] = tv;
            int ti = idx[i]; idx[i] = idx[p]; idx[p] = ti;
          }
        }
      }
      __syncthreads();
    }
  }
  const int grp = L.group[d];
  for (int iV = threadIdx.x; iV < L.nView; iV += blockDim.x)
    L.tmp[(size_t)iV * L.nDet + grp] = (float)lin_interp(key, val, L.nView, L.thetaOut[iV]);
}

__global__ void __launch_bounds__(256) rebin_t_kernel(RebinLaunch L) {
  const int iV = blockIdx.x;
  const float* row = L.tmp + (size_t)iV * L.nDet;
  for (int iD = threadIdx.x; iD < L.nDet; iD += blockDim.x)
    L.out[(size_t)iV * L.outPitch + iD] = (float)lin_interp(L.tSorted, row, L.nDet, L.posOut[iD]);
}

size_t rebin_sort_bytes(int nView) {
  int n = 1;
  while (n < nView) n <<= 1;
  return (size_t)n * (sizeof(double) + sizeof(float) + sizeof(int));
}

cudaError_t launch_rebin(RebinLaunch L, cudaStream_t s) {
  if (L.nView <= 0 || L.nDet <= 0) return cudaSuccess;
  int n = 1;
  while (n < L.nView) n <<= 1;
  L.sortN = n;
  const size_t smem = rebin_sort_bytes(L.nView);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(rebin_theta_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  rebin_theta_kernel<<<L.nDet, 256, smem, s>>>(L);
  rebin_t_kernel<<<L.nView, 256, 0, s>>>(L);
  return cudaGetLastError();
}

}  // namespace ctgpu
