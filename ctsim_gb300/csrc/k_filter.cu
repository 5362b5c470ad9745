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

// M = N / (8 blockDim) (1 or 2) and the block's thread limit are template
// parameters, so that each kernel holds only the registers its passes use
template <int M, int MAXT>
__global__ void __launch_bounds__(MAXT) fft_filter_kernel(FilterLaunch L) {
  extern __shared__ float2 zb[];   // swizzled: element m at zb[fpad<M>(m)]
  const int N = L.fftN, n = L.nDet;
  const int v0 = 2 * blockIdx.x;
  const bool two = v0 + 1 < L.nViews;
  const float* ia = L.in + (size_t)blockIdx.y * L.inSliceStride + (size_t)v0 * L.inPitch;
  const float* ib = ia + L.inPitch;
#pragma unroll 4
  for (int m = threadIdx.x; m < N; m += blockDim.x) {
    float2 v = make_float2(0.f, 0.f);
    if (m < n) {
      const float w = L.weights[m];
      v.x = w * ia[m];
      if (two) v.y = w * ib[m];
    }
    zb[fpad<M>(m)] = v;
  }
  __syncthreads();
  fft_forward_m<M>(zb, N, L.twiddle);
  // multiply by the kernel's spectrum; conjugate, so that the forward
  // transform below is the inverse one
  for (int m = threadIdx.x; m < N; m += blockDim.x) {
    const float2 z = cmul(zb[fpad<M>(m)], __ldg(&L.spectrum[m]));
    zb[fpad<M>(m)] = make_float2(z.x, -z.y);
  }
  __syncthreads();
  fft_forward_m<M>(zb, N, L.twiddle);
  float* oa = L.out + (size_t)blockIdx.y * L.outSliceStride + (size_t)v0 * L.outPitch;
  float* ob = oa + L.outPitch;
  for (int m = threadIdx.x; m < n; m += blockDim.x) {
    const float2 y = zb[fpad<M>(m)];
    oa[m] = y.x;
    if (two) ob[m] = -y.y;
  }
}

cudaError_t launch_filter(const FilterLaunch& L, cudaStream_t s) {
  if (L.nViews <= 0) return cudaSuccess;
  const int N = L.fftN;
  if (N < 4 || (N & (N - 1)) || N > 16384 || N < 2 * L.nDet - 1) return cudaErrorInvalidValue;
  const size_t smem = sizeof(float2) * (size_t)fft_smem_elems(N);
#ifndef CTGPU_FILTER_WIDE
#define CTGPU_FILTER_WIDE 16   // threads per block = N / CTGPU_FILTER_WIDE (two butterflies each)
#endif
  const int nBatch = L.nBatch > 0 ? L.nBatch : 1;
  if (nBatch > 65535) return cudaErrorInvalidConfiguration;
  const long long blocks = (long long)((L.nViews + 1) / 2) * nBatch;
  // where allowed, a launch of fewer blocks than the SMs hold at four each
  // (a single slice) gives each transform N / 8 threads: the blocks are then
  // short, and the launch is as long as one block
  static const int sms = [] {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      n = 1;
    return n;
  }();
  int T = N / (L.narrowOk && blocks < 4LL * sms ? 8 : CTGPU_FILTER_WIDE);
  if (T < 32) T = 32;
  if (T > 1024) T = 1024;
  const bool one = T * 8 >= N;
  // the radix-16 passes (M = 2) want about 70 registers: a block limit of 256
  // threads lets the compiler keep them; larger limits only where needed
  auto kern = one ? (T > 512 ? fft_filter_kernel<1, 1024>
                     : T > 256 ? fft_filter_kernel<1, 512> : fft_filter_kernel<1, 256>)
                  : (T > 512 ? fft_filter_kernel<2, 1024>
                     : T > 256 ? fft_filter_kernel<2, 512> : fft_filter_kernel<2, 256>);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  dim3 grid((L.nViews + 1) / 2, nBatch);
  kern<<<grid, T, smem, s>>>(L);
  return cudaGetLastError();
}

}  // namespace ctgpu
