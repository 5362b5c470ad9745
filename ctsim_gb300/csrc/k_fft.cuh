// k_fft.cuh -- power-of-two complex FFT of a sequence in shared memory
// (radix-8 Stockham passes, then one radix-4 or radix-2 pass), for the kernels
// of k_filter.cu and k_fourier.cu.  Each pass reads its butterflies into
// registers, synchronises, and writes them back in the next pass's order;
// twiddles come from an FP64-computed table tw[m] = exp(-2 pi i m / N).
// All threads of the block take part; blockDim >= N / 16.
//
// Element m of the sequence lives at buf[fpad<M>(m)], its low four index bits
// XORed with the next four (bits 3-6 when the first pass is radix 8, 4-7 when
// it is radix 16): a permutation within each block of 16 elements under which
// every pass's reads and writes of a half-warp fall on 16 different bank
// pairs (the first pass writes with a stride of 8 or 16 elements, which would
// otherwise hit two).  Shared memory: fft_smem_elems(N) float2.
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

// forward DFTs of length 2, 4, 8, 16 in registers, natural order in (and out,
// but for radix 16: see dft_out_index)
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
// natural output index of register r after dft<R> (radix 16 leaves its
// outputs transposed, which saves the copy)
template <int R>
__host__ __device__ constexpr int dft_out_index(int r) {
  return R == 16 ? ((r & 3) << 2) + (r >> 2) : r;
}

template <int R>
__device__ __forceinline__ void dft(float2 (&u)[R]) {
  if constexpr (R == 2) {
    dft2(u[0], u[1]);
  } else if constexpr (R == 4) {
    dft4(u[0], u[1], u[2], u[3]);
  } else if constexpr (R == 16) {
    // 4 x 4: with n = n1 + 4 n2 and k = 4 k1 + k2, X[k] is the length-4 DFT
    // over n1 of W16^(n1 k2) times the length-4 DFT over n2 of x[n1 + 4 n2]
    constexpr float c1 = 0.92387953251128676f, s1 = 0.38268343236508977f;
    constexpr float h = 0.70710678118654752f;
#pragma unroll
    for (int n1 = 0; n1 < 4; n1++) dft4(u[n1], u[n1 + 4], u[n1 + 8], u[n1 + 12]);
    // u[n1 + 4 k2] *= W16^(n1 k2), W16^j = exp(-2 pi i j / 16)
    const float2 w1 = make_float2(c1, -s1), w2 = make_float2(h, -h), w3 = make_float2(s1, -c1);
    const float2 w6 = make_float2(-h, -h), w9 = make_float2(-c1, s1);
    u[5] = cmul(u[5], w1);
    u[6] = cmul(u[6], w2);
    u[7] = cmul(u[7], w3);
    u[9] = cmul(u[9], w2);
    u[10] = mul_mi(u[10]);
    u[11] = cmul(u[11], w6);
    u[13] = cmul(u[13], w3);
    u[14] = cmul(u[14], w6);
    u[15] = cmul(u[15], w9);
#pragma unroll
    for (int k2 = 0; k2 < 4; k2++) dft4(u[4 * k2], u[4 * k2 + 1], u[4 * k2 + 2], u[4 * k2 + 3]);
    // X[4 k1 + k2] is left in u[k1 + 4 k2] (dft_out_index gives the order)
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

template <int M>
__host__ __device__ __forceinline__ int fpad(int m) { return m ^ ((m >> (M == 2 ? 4 : 3)) & 15); }
// the same with M known only at run time (fft_forward's choice)
__device__ __forceinline__ int fft_swizzle_shift(int N) { return (int)blockDim.x * 8 >= N ? 3 : 4; }
__device__ __forceinline__ int fpad_rt(int m, int sh) { return m ^ ((m >> sh) & 15); }
__host__ __device__ __forceinline__ int fft_smem_elems(int n) { return (n + 15) & ~15; }

// One Stockham pass of radix R over buf[N] (p = product of the radices done):
// butterfly i takes x[i + r N/R], twiddles by W^(r k N/(pR)) with k = i mod p,
// and writes y[(i - k) R + k + r p].
// M = N / (8 blockDim) (1 or 2): butterflies per thread M * 8 / R (radix 16
// only with M = 2).
template <int R, int M>
__device__ __forceinline__ void stockham_pass(float2* buf, int N, int p,
                                              const float2* __restrict__ tw) {
  static_assert(M * 8 >= R, "radix 16 needs blockDim <= N / 16");
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
        float2 v = buf[fpad<M>(i + r * nb)];
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
      for (int r = 0; r < R; r++) buf[fpad<M>(j + dft_out_index<R>(r) * p)] = u[s][r];
    }
  }
  __syncthreads();
}

// M == 2 (blockDim = N / 16) runs radix-16 passes (one butterfly per thread)
// while they fit, fewer passes through shared memory
template <int M>
__device__ void fft_forward_m(float2* buf, int N, const float2* __restrict__ tw) {
  int p = 1;
  if constexpr (M == 2)
    while (p * 16 <= N) {
      stockham_pass<16, M>(buf, N, p, tw);
      p *= 16;
    }
  while (p * 8 <= N) {
    stockham_pass<8, M>(buf, N, p, tw);
    p *= 8;
  }
  if (p * 4 == N) stockham_pass<4, M>(buf, N, p, tw);
  else if (p * 2 == N) stockham_pass<2, M>(buf, N, p, tw);
}

// forward transform of buf (layout fpad_rt(m, fft_swizzle_shift(N))); blockDim >= N / 16
__device__ __forceinline__ void fft_forward(float2* buf, int N, const float2* __restrict__ tw) {
  if ((int)blockDim.x * 8 >= N) fft_forward_m<1>(buf, N, tw);
  else fft_forward_m<2>(buf, N, tw);
}

}  // namespace
}  // namespace ctgpu
