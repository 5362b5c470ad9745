// k_fft.cuh -- power-of-two complex FFT of a sequence in shared memory
// (radix-8 Stockham passes, then one radix-4 or radix-2 pass), for the kernels
// of k_filter.cu and k_fourier.cu.  Each pass reads its butterflies into
// registers, synchronises, and writes them back in the next pass's order;
// twiddles come from an FP64-computed table tw[m] = exp(-2 pi i m / N).
// All threads of the block take part; blockDim >= N / 16.
//
// Element m of the sequence lives at buf[fpad(m)], its low four index bits
// XORed with bits 3-6 (a permutation within each block of 16 elements): every
// pass's reads and writes of a half-warp then fall on 16 different bank pairs
// (the first pass writes with a stride of 8 elements, which would otherwise
// hit two).  Shared memory: fft_smem_elems(N) float2.
#pragma once

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

__host__ __device__ __forceinline__ int fpad(int m) { return m ^ ((m >> 3) & 15); }
__host__ __device__ __forceinline__ int fft_smem_elems(int n) { return (n + 15) & ~15; }

// One Stockham pass of radix R over buf[N] (p = product of the radices done):
// butterfly i takes x[i + r N/R], twiddles by W^(r k N/(pR)) with k = i mod p,
// and writes y[(i - k) R + k + r p].
// M = N / (8 blockDim) (1 or 2): butterflies per thread M * 8 / R.
template <int R, int M>
__device__ __forceinline__ void stockham_pass(float2* buf, int N, int p,
                                              const float2* __restrict__ tw) {
  constexpr int SMAX = M * 8 / R;
  const int nb = N / R, T = blockDim.x, stride = N / (p * R);
  float2 u[SMAX][R];
#pragma unroll
  for (int s = 0; s < SMAX; s++) {
    const int i = threadIdx.x + s * T;
    if (i < nb) {
      const int k = i & (p - 1);
#pragma unroll
      for (int r = 0; r < R; r++) {
        float2 v = buf[fpad(i + r * nb)];
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
      for (int r = 0; r < R; r++) buf[fpad(j + r * p)] = u[s][r];
    }
  }
  __syncthreads();
}

template <int M>
__device__ void fft_forward_m(float2* buf, int N, const float2* __restrict__ tw) {
  int p = 1;
  while (p * 8 <= N) {
    stockham_pass<8, M>(buf, N, p, tw);
    p *= 8;
  }
  if (p * 4 == N) stockham_pass<4, M>(buf, N, p, tw);
  else if (p * 2 == N) stockham_pass<2, M>(buf, N, p, tw);
}

// forward transform of buf (padded layout); blockDim >= N / 16
__device__ __forceinline__ void fft_forward(float2* buf, int N, const float2* __restrict__ tw) {
  if ((int)blockDim.x * 8 >= N) fft_forward_m<1>(buf, N, tw);
  else fft_forward_m<2>(buf, N, tw);
}

}  // namespace
}  // namespace ctgpu
