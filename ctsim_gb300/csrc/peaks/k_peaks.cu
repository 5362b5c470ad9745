// k_peaks.cu -- measured roofline denominators for the benchmark (libctpeaks.so).
//
// The backprojection's per-pixel-view work is FP32 arithmetic on rows staged in
// shared memory; its rate is reported as a fraction of the FP32 FMA peak and
// of the gather bandwidth (shared memory and L2).  This library measures
// those peaks on the GPU it runs on, with CUDA events, best of several
// launches:
//
//   out[0]  scalar FFMA throughput, TFLOP/s (FMA = 2 FLOP), 8 independent
//           chains per thread, 4 CTAs x 256 threads per SM
//   out[1]  packed FFMA2 throughput (two FP32 FMAs per instruction), TFLOP/s
//   out[2]  shared-memory LDS.128 bandwidth, GB/s: each warp reads 32
//           consecutive 16-byte words (no bank conflicts), 4 CTAs per SM
//   out[3]  16-byte gathers from an L2-resident 16 MiB buffer at pseudo-random
//           positions, GB/s of bytes delivered to the threads (ld.global.cg)
//   out[4]  coalesced 16-byte reads of the same L2-resident buffer, GB/s
//   out[5]  SM count used
//
// Every kernel folds what it loads or computes into a value that is written
// only under a condition the data never meets, so nothing is optimised away
// and nothing is written.  All indexes are masked into their buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

namespace {

constexpr int kThreads = 256;
constexpr int kCtasPerSm = 4;

__global__ void __launch_bounds__(kThreads) ffma_kernel(float* sink, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
  float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
  }
  float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == -1.2345e30f) sink[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) ffma2_kernel(float* sink, int iters, float a, float b) {
  const float2 av = make_float2(a, a), bv = make_float2(b, b);
  float2 x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = make_float2(threadIdx.x * 1e-3f + k, threadIdx.x * 2e-3f + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++) {
#pragma unroll
      for (int k = 0; k < 8; k++) x[k] = __ffma2_rn(x[k], av, bv);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k].x + x[k].y;
  if (s == -1.2345e30f) sink[blockIdx.x] = s;
}

constexpr int kLdsWords = 2048;   // 16-byte words, 32 KB per CTA

__global__ void __launch_bounds__(kThreads) lds128_kernel(float* sink, int iters) {
  __shared__ float4 buf[kLdsWords];
  for (int i = threadIdx.x; i < kLdsWords; i += kThreads)
    buf[i] = make_float4(i * 1e-3f, i * 2e-3f, i * 3e-3f, i * 4e-3f);
  __syncthreads();
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  const int base = threadIdx.x;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const float4 v = buf[(base + u * kThreads + i * 32) & (kLdsWords - 1)];
      acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
    }
  }
  float s = (acc.x + acc.y) + (acc.z + acc.w);
  if (s == -1.2345e30f) sink[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) l2_gather_kernel(const float4* __restrict__ buf,
                                                             unsigned mask, int iters, float* sink) {
  unsigned h = (blockIdx.x * kThreads + threadIdx.x) * 2654435761u + 12345u;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++) {
      h = h * 1664525u + 1013904223u;
      const float4 v = __ldcg(buf + ((h >> 7) & mask));
      acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
    }
  }
  float s = (acc.x + acc.y) + (acc.z + acc.w);
  if (s == -1.2345e30f) sink[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) l2_read_kernel(const float4* __restrict__ buf,
                                                           unsigned mask, int iters, float* sink) {
  const unsigned stride = gridDim.x * kThreads;
  unsigned p = blockIdx.x * kThreads + threadIdx.x;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 8; u++) {
      const float4 v = __ldcg(buf + (p & mask));
      p += stride;
      acc.x += v.x; acc.y += v.y; acc.z += v.z; acc.w += v.w;
    }
  }
  float s = (acc.x + acc.y) + (acc.z + acc.w);
  if (s == -1.2345e30f) sink[blockIdx.x] = s;
}

__global__ void fill_kernel(float4* buf, unsigned n) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    buf[i] = make_float4(i * 1e-6f, 1.f, 2.f, 3.f);
}

template <typename F>
float best_ms(F launch, cudaStream_t s, int reps, cudaError_t* err) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  launch();   // warm-up
  float best = 1e30f;
  for (int r = 0; r < reps; r++) {
    cudaEventRecord(a, s);
    launch();
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    best = std::min(best, ms);
  }
  *err = cudaGetLastError();
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

}  // namespace

extern "C" int ctpeaks_measure(double* out, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return 1;
  const int grid = sms * kCtasPerSm;
  const double threads = (double)grid * kThreads;
  float* sink = nullptr;
  float4* buf = nullptr;
  const unsigned words = 1u << 20;   // 16 MiB, well inside L2
  if (cudaMalloc(&sink, sizeof(float) * grid) != cudaSuccess) return 1;
  if (cudaMalloc(&buf, sizeof(float4) * words) != cudaSuccess) { cudaFree(sink); return 1; }
  const int reps = 5;
  cudaError_t err = cudaSuccess;

  const int fIters = 4096;
  float ms = best_ms([&] { ffma_kernel<<<grid, kThreads, 0, s>>>(sink, fIters, 0.9999f, 1e-7f); },
                     s, reps, &err);
  out[0] = threads * fIters * 16 * 8 * 2 / (ms * 1e-3) / 1e12;
  if (err == cudaSuccess)
    ms = best_ms([&] { ffma2_kernel<<<grid, kThreads, 0, s>>>(sink, fIters, 0.9999f, 1e-7f); },
                 s, reps, &err);
  out[1] = threads * fIters * 8 * 8 * 2 * 2 / (ms * 1e-3) / 1e12;
  const int lIters = 4096;
  if (err == cudaSuccess)
    ms = best_ms([&] { lds128_kernel<<<grid, kThreads, 0, s>>>(sink, lIters); }, s, reps, &err);
  out[2] = threads * lIters * 8 * 16 / (ms * 1e-3) / 1e9;
  if (err == cudaSuccess) {
    fill_kernel<<<grid, kThreads, 0, s>>>(buf, words);
    err = cudaGetLastError();
  }
  const int gIters = 1024;
  if (err == cudaSuccess)
    ms = best_ms([&] { l2_gather_kernel<<<grid, kThreads, 0, s>>>(buf, words - 1, gIters, sink); },
                 s, reps, &err);
  out[3] = threads * gIters * 8 * 16 / (ms * 1e-3) / 1e9;
  if (err == cudaSuccess)
    ms = best_ms([&] { l2_read_kernel<<<grid, kThreads, 0, s>>>(buf, words - 1, gIters, sink); },
                 s, reps, &err);
  out[4] = threads * gIters * 8 * 16 / (ms * 1e-3) / 1e9;
  out[5] = sms;
  cudaStreamSynchronize(s);
  cudaFree(buf);
  cudaFree(sink);
  return err == cudaSuccess ? 0 : 1;
}
