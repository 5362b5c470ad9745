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
// FFT: k_fft.cuh's shared-memory Stockham transform.  One CTA per view pair
// and slice.
#include "k_fft.cuh"

namespace ctgpu {

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
