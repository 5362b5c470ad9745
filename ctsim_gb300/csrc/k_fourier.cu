// k_fourier.cu -- polar and direct-Fourier images on sm_103a.
//
// Projections::convertPolar and ::convertFFTPolar (libctsim/projections.cpp:
// 953-1180) and the GUI's Fourier reconstruction (src/views.cpp:2828-2849):
// convertFFTPolar, then ImageFile::ifft (libctsim/imagefile.cpp:770-826),
// magnitude (:1175-1198) and Fourier::shuffleFourierToNaturalOrder
// (libctsim/fourier.cpp:31-63).
//
// polar_kernel: one thread per pixel.  The pixel's polar coordinates
// (calcArrayPolarCoordinates, :1113-1149) and the nearest / bilinear polar
// interpolation (interpolatePolar, :1136-1180; BilinearPolarInterpolator,
// include/interpolator.h:92-154) are FP64 as in the reference; the pixel
// centres come from the host, accumulated by the reference's own additions.
//
// fourier_views_kernel: one CTA per view.  The view is interpolated to
// nInterp points, shifted so its middle sits at index 0, zero padded in the
// middle to N points, transformed (FFTW_FORWARD's sign) and shifted back --
// all in shared memory.  Power-of-two N use k_fft.cuh's Stockham transform;
// other N a direct DFT with exact twiddle indices (j k mod N).
//
// ifft_lines_kernel: the backward 2-D DFT as two passes of line transforms
// (along y, then along x); the second pass also takes the FP32 magnitude and
// writes the result in natural order.  Both index shuffles are gathers.
#include "k_fft.cuh"

namespace ctgpu {

namespace {

// Fourier::shuffleFourierToNaturalOrder: new[d] = old[nat_src(n, d)]
__device__ __forceinline__ int nat_src(int n, int d) {
  if (n & 1) {
    const int h = (n - 1) / 2;
    return d == h ? 0 : (d > h ? d - h : d + h + 1);
  }
  const int h = n / 2;
  return d == h ? 0 : (d < h ? d + h : d - h);
}
// Fourier::shuffleNaturalToFourierOrder: new[d] = old[fou_src(n, d)]
__device__ __forceinline__ int fou_src(int n, int d) {
  if (n & 1) {
    const int h = (n - 1) / 2;
    return d == 0 ? h : (d <= h ? d + h : d - h - 1);
  }
  const int h = n / 2;
  return d == 0 ? h : (d < h ? d + h : d - h);
}

// the value of a polar data set at (view, position), one component
struct PolarData {
  const float* re;    // [nAngle][pitch] floats (real data) or float2 pairs
  bool complexData;   // float2 [nAngle][pitch]
  int pitch;
  __device__ __forceinline__ double get(int a, int p, int comp) const {
    if (!complexData) return comp == 0 ? (double)re[(size_t)a * pitch + p] : 0.0;
    return (double)re[2 * ((size_t)a * pitch + p) + comp];
  }
};

// BilinearPolarInterpolator::interpolate of one component
__device__ double bilinear_polar(const PolarData& m, int comp, int nAngle, int nPos,
                                 double dAngle, double dPos) {
  const int fa0 = (int)floor(dAngle), fp0 = (int)floor(dPos);
  const double fa = dAngle - fa0, fp = dPos - fp0;
  if (fa0 < -1 || fp0 < 0 || fa0 > nAngle - 1 || fp0 > nPos - 1) return 0.0;
  if (fa0 == -1 && fp0 == nPos - 1)
    return m.get(0, nPos - 1, comp) + fa * (m.get(nAngle - 1, fp0, comp) - m.get(0, fp0, comp));
  if (fa0 == nAngle - 1 && fp0 == nPos - 1)
    return m.get(nAngle - 1, nPos - 1, comp) +
           fa * (m.get(0, fp0, comp) - m.get(nAngle - 1, fp0, comp));
  if (fp0 == nPos - 1)
    return m.get(fa0, fp0, comp) + fa * (m.get(fa0 + 1, fp0, comp) - m.get(fa0, fp0, comp));
  // the general case and the two wrap-arounds in angle (the position mirrors)
  int a0 = fa0, a1 = fa0 + 1, p00 = fp0, p01 = fp0 + 1, p10 = fp0, p11 = fp0 + 1;
  if (fa0 == nAngle - 1) {
    a1 = 0;
    p10 = (nPos - 1) - fp0;
    p11 = (nPos - 1) - (fp0 + 1);
  } else if (fa0 == -1) {
    a0 = nAngle - 1;
    p00 = (nPos - 1) - fp0;
    p01 = (nPos - 1) - (fp0 + 1);
  }
  return (1 - fa) * (1 - fp) * m.get(a0, p00, comp) + fa * (1 - fp) * m.get(a1, p10, comp) +
         fp * (1 - fa) * m.get(a0, p01, comp) + fa * fp * m.get(a1, p11, comp);
}

// one thread per pixel of columns < cols (= min(nx, ny): the reference's
// interpolatePolar loops ix over ny); later columns are zeroed
__global__ void __launch_bounds__(256) polar_kernel(PolarLaunch L) {
  const int ix = blockIdx.y, iy = blockIdx.x * blockDim.x + threadIdx.x;
  if (iy >= L.ny) return;
  const size_t o = (size_t)ix * L.ny + iy;
  double vr = 0.0, vi = 0.0;
  if (ix < L.cols) {
    const double x = L.xs[ix], y = L.ys[iy];
    double r = sqrt(x * x + y * y);
    double phi = atan2(y, x);
    if (phi <= -L.rotInc / 2) phi += kTwoPi;
    if (phi >= kPi - (L.rotInc / 2)) {
      phi -= kPi;
      r = -r;
    }
    const double dView = (phi - L.rotStart) / L.rotInc;
    const double dDet = (r / L.detInc) + L.detCenter;
    const PolarData m{L.data, L.complexData != 0, L.pitch};
    if (L.interp == 0) {
      unsigned int iv = (unsigned int)(dView > 0 ? (int)(dView + 0.5) : (int)(dView - 0.5));
      const unsigned int id = (unsigned int)(dDet > 0 ? (int)(dDet + 0.5) : (int)(dDet - 0.5));
      if (iv == (unsigned int)L.nView) iv = 0;
      if (id < (unsigned int)L.nPos && iv < (unsigned int)L.nView) {
        vr = m.get(iv, id, 0);
        vi = m.get(iv, id, 1);
      }
    } else {
      vr = bilinear_polar(m, 0, L.nView, L.nPos, dView, dDet);
      if (L.complexData) vi = bilinear_polar(m, 1, L.nView, L.nPos, dView, dDet);
    }
  }
  L.outRe[o] = (float)vr;
  if (L.outIm) L.outIm[o] = (float)vi;
}

// direct DFT of z (swizzled layout, element j at z[fpad_rt(j, sh)]; sign -1 forward,
// +1 backward) into out[n] (plain layout), shared memory
__device__ void dft_direct(const float2* z, float2* out, int n, const float2* __restrict__ tw,
                           int sign, int sh) {
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    float sr = 0.f, si = 0.f;
    int idx = 0;   // j k mod n, advanced by k
    for (int j = 0; j < n; j++) {
      const float2 w = __ldg(&tw[idx]);
      const float wi = sign < 0 ? w.y : -w.y;
      const float2 zj = z[fpad_rt(j, sh)];
      sr = fmaf(zj.x, w.x, fmaf(-zj.y, wi, sr));
      si = fmaf(zj.x, wi, fmaf(zj.y, w.x, si));
      idx += k;
      if (idx >= n) idx -= n;
    }
    out[k] = make_float2(sr, si);
  }
}

// transform buf (swizzled layout) in place (pow2: Stockham; else direct DFT
// through tmp)
__device__ __forceinline__ void line_transform(float2* buf, float2* tmp, int n,
                                               const float2* __restrict__ tw, int sign, int sh) {
  if ((n & (n - 1)) == 0) {
    if (sign > 0)   // backward = conj(forward(conj))
      for (int m = threadIdx.x; m < n; m += blockDim.x) buf[fpad_rt(m, sh)].y = -buf[fpad_rt(m, sh)].y;
    __syncthreads();
    if (n > 1) fft_forward(buf, n, tw);
    if (sign > 0) {
      for (int m = threadIdx.x; m < n; m += blockDim.x) buf[fpad_rt(m, sh)].y = -buf[fpad_rt(m, sh)].y;
      __syncthreads();
    }
  } else {
    __syncthreads();
    dft_direct(buf, tmp, n, tw, sign, sh);
    __syncthreads();
    for (int m = threadIdx.x; m < n; m += blockDim.x) buf[fpad_rt(m, sh)] = tmp[m];
    __syncthreads();
  }
}

// one CTA per view: convertFFTPolar's per-view steps (projections.cpp:1034-1067)
__global__ void __launch_bounds__(1024) fourier_views_kernel(FourierViewsLaunch L) {
  extern __shared__ float2 zs[];
  float2* buf = zs;                          // swizzled layout
  float2* tmp = zs + fft_smem_elems(L.N);    // direct DFT only
  const int v = blockIdx.x, N = L.N, nI = L.nInterp, nDet = L.nDet;
  const int sh = fft_swizzle_shift(N);
  const float* row = L.sino + (size_t)v * L.pitch;
  const int zeros = N - nI;
  for (int m = threadIdx.x; m < N; m += blockDim.x) {
    int s = m;   // index into the shifted, interpolated view
    bool zero = false;
    if (zeros > 0) {
      if (m >= L.iMid && m < L.iMid + zeros) zero = true;
      else if (m >= L.iMid + zeros) s = m - zeros;
    }
    float2 val = make_float2(0.f, 0.f);
    if (!zero) {
      // LinearInterpolator<float> at x (zero outside the detector row)
      const int i = nat_src(nI, s);
      const double x = L.posTable[i];
      double r;
      if (x == 0) r = row[0];
      else if (x < 0) r = 0.0;
      else if (x == nDet - 1) r = row[nDet - 1];
      else if (x > nDet - 1) r = 0.0;
      else {
        const int f = (int)floor(x);
        r = (double)row[f] + (double)__fsub_rn(row[f + 1], row[f]) * (x - f);
      }
      val.x = (float)(r * L.projScale);
    }
    buf[fpad_rt(m, sh)] = val;
  }
  __syncthreads();
  line_transform(buf, tmp, N, L.twiddle, -1, sh);
  float2* out = L.spec + (size_t)v * N;
  const float sc = (float)L.fftScale;
  for (int d = threadIdx.x; d < N; d += blockDim.x) {
    const float2 z = buf[fpad_rt(nat_src(N, d), sh)];
    out[d] = make_float2(z.x * sc, z.y * sc);
  }
}

// backward 2-D DFT, pass 1: line ix (CTA) along y, input gathered through
// shuffleNaturalToFourierOrder; pass 2: line k2 along x, FP32 magnitude,
// written in natural order
__global__ void __launch_bounds__(1024) ifft_lines_kernel(IfftLaunch L, int pass) {
  extern __shared__ float2 zs[];
  const int nx = L.nx, ny = L.ny;
  const int n = pass == 1 ? ny : nx;
  float2* buf = zs;                      // swizzled layout
  float2* tmp = zs + fft_smem_elems(n);   // direct DFT only
  const int line = blockIdx.x;
  const int sh = fft_swizzle_shift(n);
  if (pass == 1) {
    const int sx = fou_src(nx, line);
    for (int m = threadIdx.x; m < ny; m += blockDim.x) {
      const size_t s = (size_t)sx * ny + fou_src(ny, m);
      buf[fpad_rt(m, sh)] = make_float2(L.inRe[s], L.inIm[s]);
    }
  } else {
    const int k2 = nat_src(ny, line);   // this CTA writes output row `line`
    for (int m = threadIdx.x; m < nx; m += blockDim.x) buf[fpad_rt(m, sh)] = L.tmp[(size_t)m * ny + k2];
  }
  __syncthreads();
  line_transform(buf, tmp, n, pass == 1 ? L.twY : L.twX, +1, sh);
  if (pass == 1) {
    for (int m = threadIdx.x; m < ny; m += blockDim.x) L.tmp[(size_t)line * ny + m] = buf[fpad_rt(m, sh)];
  } else {
    for (int d1 = threadIdx.x; d1 < nx; d1 += blockDim.x) {
      const float2 z = buf[fpad_rt(nat_src(nx, d1), sh)];   // the reference keeps FP32 re / im
      const float mag = __fsqrt_rn(__fadd_rn(__fmul_rn(z.x, z.x), __fmul_rn(z.y, z.y)));
      L.out[(size_t)d1 * ny + line] = mag;
    }
  }
}

int line_threads(int n) {
  int t = n / 8;
  if (t < 64) t = 64;
  if (t > 1024) t = 1024;
  return (t + 31) & ~31;
}

}  // namespace

cudaError_t launch_polar(const PolarLaunch& L, cudaStream_t s) {
  if (L.nx <= 0 || L.ny <= 0) return cudaSuccess;
  if (L.nx > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((L.ny + 255) / 256, L.nx);
  polar_kernel<<<grid, 256, 0, s>>>(L);
  return cudaGetLastError();
}

size_t line_smem_bytes(int n) {
  return sizeof(float2) * ((size_t)fft_smem_elems(n) + (((n & (n - 1)) == 0) ? 0 : (size_t)n));
}

cudaError_t launch_fourier_views(const FourierViewsLaunch& L, cudaStream_t s) {
  if (L.nView <= 0) return cudaSuccess;
  const size_t smem = line_smem_bytes(L.N);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fourier_views_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  fourier_views_kernel<<<L.nView, line_threads(L.N), smem, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_ifft_magnitude(const IfftLaunch& L, cudaStream_t s) {
  if (L.nx <= 0 || L.ny <= 0) return cudaSuccess;
  for (int pass = 1; pass <= 2; pass++) {
    const int n = pass == 1 ? L.ny : L.nx, lines = pass == 1 ? L.nx : L.ny;
    const size_t smem = line_smem_bytes(n);
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(ifft_lines_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    ifft_lines_kernel<<<lines, line_threads(n), smem, s>>>(L, pass);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace ctgpu
