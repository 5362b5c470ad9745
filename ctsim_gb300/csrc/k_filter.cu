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
// weight) and this kernel evaluates the resulting Toeplitz product in FP32
// with FP32 accumulation.  A CTA owns VB views and a strip of 4*blockDim
// outputs; the taps and the weighted input rows are staged in shared memory,
// each thread keeps 4 outputs x VB views in registers and slides a 4-tap
// window, so one shared load feeds 4*VB FMAs.
#include "ctgpu_internal.h"

namespace ctgpu {

namespace {
constexpr int VB = 8;          // views per CTA
constexpr int NT = 64;         // threads per CTA
constexpr int OUT_PER_CTA = 4 * NT;
constexpr int TPAD = 4;        // zero taps before index 0
}

__global__ void __launch_bounds__(NT) toeplitz_filter_kernel(FilterLaunch L) {
  extern __shared__ float sm[];
  const int n = L.nDet;
  const int n4 = (n + 3) & ~3;
  const int ntap = 2 * n - 1;
  const int tapLen = ntap + TPAD + 12;
  float* tp = sm;                      // tp[j + TPAD] = taps[j]
  float* xs = sm + ((tapLen + 3) & ~3);  // [VB][n4] weighted inputs
  const int v0 = blockIdx.x * VB;
  const int nv = min(VB, L.nViews - v0);
  for (int j = threadIdx.x; j < tapLen; j += NT) {
    int k = j - TPAD;
    tp[j] = (k >= 0 && k < ntap) ? L.taps[k] : 0.f;
  }
  for (int v = 0; v < VB; v++) {
    for (int i = threadIdx.x; i < n4; i += NT) {
      float x = 0.f;
      if (v < nv && i < n) x = L.weights[i] * L.in[(size_t)(v0 + v) * L.inPitch + i];
      xs[v * n4 + i] = x;
    }
  }
  __syncthreads();

  const int nOut0 = blockIdx.y * OUT_PER_CTA + 4 * threadIdx.x;
  if (nOut0 >= n) return;
  float acc[VB][4];
#pragma unroll
  for (int v = 0; v < VB; v++)
#pragma unroll
    for (int k = 0; k < 4; k++) acc[v][k] = 0.f;

  // window w[k] = taps[nOut0 + k - i + n - 1]
  int base = nOut0 + n - 1 + TPAD;   // smem index of taps[nOut0 - 0 + n - 1]
  float w0 = tp[base], w1 = tp[base + 1], w2 = tp[base + 2], w3 = tp[base + 3];
  for (int i = 0; i < n4; i += 4) {
    float4 xv[VB];
#pragma unroll
    for (int v = 0; v < VB; v++) xv[v] = *reinterpret_cast<const float4*>(&xs[v * n4 + i]);
#pragma unroll
    for (int q = 0; q < 4; q++) {
#pragma unroll
      for (int v = 0; v < VB; v++) {
        float xq = q == 0 ? xv[v].x : q == 1 ? xv[v].y : q == 2 ? xv[v].z : xv[v].w;
        acc[v][0] = fmaf(xq, w0, acc[v][0]);
        acc[v][1] = fmaf(xq, w1, acc[v][1]);
        acc[v][2] = fmaf(xq, w2, acc[v][2]);
        acc[v][3] = fmaf(xq, w3, acc[v][3]);
      }
      // slide: next input index uses taps shifted down by one
      w3 = w2; w2 = w1; w1 = w0;
      w0 = tp[base - (i + q + 1)];
    }
  }
#pragma unroll
  for (int v = 0; v < VB; v++) {
    if (v >= nv) break;
    float* o = L.out + (size_t)(v0 + v) * L.outPitch;
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (nOut0 + k < n) o[nOut0 + k] = acc[v][k];
  }
}

cudaError_t launch_filter(const FilterLaunch& L, cudaStream_t s) {
  if (L.nViews <= 0) return cudaSuccess;
  const int n = L.nDet;
  const int n4 = (n + 3) & ~3;
  const int tapLen = 2 * n - 1 + TPAD + 12;
  size_t smem = sizeof(float) * (size_t)(((tapLen + 3) & ~3) + VB * n4);
  if (smem > 220 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(toeplitz_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
  dim3 grid((L.nViews + VB - 1) / VB, (n + OUT_PER_CTA - 1) / OUT_PER_CTA);
  toeplitz_filter_kernel<<<grid, NT, smem, s>>>(L);
  return cudaGetLastError();
}

}  // namespace ctgpu
