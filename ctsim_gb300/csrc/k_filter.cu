// k_filter.cu -- projection filtering on sm_103a.
//
// Every filter method of ProcessSignal::filterSignal (libctsim/procsignal.cpp:
// 543-629) is a linear, shift-invariant map of one view's nDet samples:
//   convolution   out[n] = dx * sum_i in[i] h[n - i + nDet - 1]      (:658-691)
//   fourier / fouier-table / fft (zero padded to N, frequency filter H)
//                 out[n] = sum_i in[i] c[(n - i) mod N],
//                 c[m] = (1/N) sum_k H[k] cos(2 pi k m / N)          (:565-626)
// so the host folds the chosen filter into one tap vector of length
// 2 nDet - 1 in FP64 (the fan pre-weighting of :551-561 becomes a per-sample
// weight), and from it the DFT of the equivalent circular kernel of length
// fftN >= 2 nDet - 1 (no lag wraps around).  This kernel evaluates the
// convolution as FFT -> multiply -> inverse FFT in FP32, two views at a time:
// view a in the real part, view b in the imaginary part of one complex
// sequence.  The kernel is real, so its spectrum is Hermitian and the
// product keeps the two views apart: the real part of the result is a's
// output, the imaginary part b's.  The inverse transform is the forward one
// on the conjugate.
//
// FFT: radix-8 Stockham passes (then one radix-4 or radix-2 pass) on the
// sequence in shared memory; each pass reads its butterflies into registers,
// synchronises, and writes them back in the next pass's order.  Twiddles come
// from an FP64-computed table.  One CTA per view pair and slice.
#include "ctgpu_internal.h"

namespace ctgpu {

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// times -i
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }

// forward DFTs of length 2, 4, 8 in registers, natural order in and out
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  const float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3) {
  const float2 s0 = cadd(a0, a2), s1 = csub(a0, a2);
  const float2 s2 = cadd(a1, a3), s3 = mul_mi(csub(a1, a3));
  a0 = cadd(s0, s2);
  a2 = csub(s0, s2);
  a1 = cadd(s1, s3);
  a3 = csub(s1, s3);
}
template <int R>
__device__ __forceinline__ void dft(float2 (&u)[R]) {
  if constexpr (R == 2) {
    dft2(u[0], u[1]);
  } else if constexpr (R == 4) {
    dft4(u[0], u[1], u[2], u[3]);
  } else {
    // radix 2 x 4: even outputs from the sums, odd ones from the twiddled
    // differences (w8 = exp(-i pi / 4))
    constexpr float c = 0.70710678118654752f;
    float2 a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      a[r] = cadd(u[r], u[r + 4]);
      b[r] = csub(u[r], u[r + 4]);
    }
    b[1] = make_float2(c * (b[1].x + b[1].y), c * (b[1].y - b[1].x));
    b[2] = mul_mi(b[2]);
    b[3] = make_float2(c * (b[3].y - b[3].x), -c * (b[3].x + b[3].y));
    dft4(a[0], a[1], a[2], a[3]);
    dft4(b[0], b[1], b[2], b[3]);
#pragma unroll
    for (int k = 0; k < 4; k++) {
      u[2 * k] = a[k];
      u[2 * k + 1] = b[k];
    }
  }
}

// One Stockham pass of radix R over buf[N] (p = product of the radices done):
// butterfly i takes x[i + r N/R], twiddles by W^(r k N/(pR)) with k = i mod p,
// and writes y[(i - k) R + k + r p].
template <int R>
__device__ __forceinline__ void stockham_pass(float2* buf, int N, int p,
                                              const float2* __restrict__ tw) {
  constexpr int SMAX = 16 / R;   // butterflies per thread (blockDim >= N / 8)
  const int nb = N / R, T = blockDim.x, stride = N / (p * R);
  float2 u[SMAX][R];
#pragma unroll
  for (int s = 0; s < SMAX; s++) {
    const int i = threadIdx.x + s * T;
    if (i < nb) {
      const int k = i & (p - 1);
#pragma unroll
      for (int r = 0; r < R; r++) {
        float2 v = buf[i + r * nb];
        if (r > 0 && k > 0) v = cmul(v, __ldg(&tw[r * k * stride]));
        u[s][r] = v;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int s = 0; s < SMAX; s++) {
    const int i = threadIdx.x + s * T;
    if (i < nb) {
      const int k = i & (p - 1);
      dft<R>(u[s]);
      const int j = (i - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; r++) buf[j + r * p] = u[s][r];
    }
  }
  __syncthreads();
}

__device__ void fft_forward(float2* buf, int N, const float2* __restrict__ tw) {
  int p = 1;
  while (p * 8 <= N) {
    stockham_pass<8>(buf, N, p, tw);
    p *= 8;
  }
  if (p * 4 == N) stockham_pass<4>(buf, N, p, tw);
  else if (p * 2 == N) stockham_pass<2>(buf, N, p, tw);
}

}  // namespace

__global__ void __launch_bounds__(1024) fft_filter_kernel(FilterLaunch L) {
  extern __shared__ float2 zb[];
  const int N = L.fftN, n = L.nDet;
  const int v0 = 2 * blockIdx.x;
  const bool two = v0 + 1 < L.nViews;
  const float* ia = L.in + (size_t)blockIdx.y * L.inSliceStride + (size_t)v0 * L.inPitch;
  const float* ib = ia + L.inPitch;
  for (int m = threadIdx.x; m < N; m += blockDim.x) {
    float2 v = make_float2(0.f, 0.f);
    if (m < n) {
      const float w = L.weights[m];
      v.x = w * ia[m];
      if (two) v.y = w * ib[m];
    }
    zb[m] = v;
  }
  __syncthreads();
  fft_forward(zb, N, L.twiddle);
  // multiply by the kernel's spectrum; conjugate, so that the forward
  // transform below is the inverse one
  for (int m = threadIdx.x; m < N; m += blockDim.x) {
    const float2 z = cmul(zb[m], __ldg(&L.spectrum[m]));
    zb[m] = make_float2(z.x, -z.y);
  }
  __syncthreads();
  fft_forward(zb, N, L.twiddle);
  float* oa = L.out + (size_t)blockIdx.y * L.outSliceStride + (size_t)v0 * L.outPitch;
  float* ob = oa + L.outPitch;
  for (int m = threadIdx.x; m < n; m += blockDim.x) {
    const float2 y = zb[m];
    oa[m] = y.x;
    if (two) ob[m] = -y.y;
  }
}

cudaError_t launch_filter(const FilterLaunch& L, cudaStream_t s) {
  if (L.nViews <= 0) return cudaSuccess;
  const int N = L.fftN;
  if (N < 4 || (N & (N - 1)) || N > 16384 || N < 2 * L.nDet - 1) return cudaErrorInvalidValue;
  const size_t smem = sizeof(float2) * (size_t)N;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(fft_filter_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int T = N / 8;
  if (T < 32) T = 32;
  if (T > 1024) T = 1024;
  const int nBatch = L.nBatch > 0 ? L.nBatch : 1;
  if (nBatch > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((L.nViews + 1) / 2, nBatch);
  fft_filter_kernel<<<grid, T, smem, s>>>(L);
  return cudaGetLastError();
}

}  // namespace ctgpu
