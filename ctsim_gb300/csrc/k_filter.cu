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
// Two kernels:
//   fft_filter_persistent_kernel (batched launches, fftN 512 .. 4096): a
//     persistent grid, each block looping over view pairs with its twiddle
//     factors held in registers and the next pair's rows on their way into
//     shared memory (cp.async) while it transforms the current one; it can
//     also write the interval rows of the table-family backprojection straight
//     from its output;
//   fft_filter_kernel (one CTA per view pair and slice; the single-slice
//     launches of few blocks, and fftN 8192 and 16384, whose sequences
//     need dynamic shared memory): k_fft.cuh's shared-memory
//     Stockham transform; it writes the interval rows too where asked.
#include <algorithm>
#include <cstdint>

#include "k_fft.cuh"
#include "k_rows.cuh"

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
  // the interval rows of both views, as the persistent kernel writes them
  if (L.rows) {
    const int rp = L.rowsPitch;
    const size_t rbase = (size_t)blockIdx.y * L.rowsSliceStride + (size_t)v0 * rp;
    const float2* zs = zb;
    auto fa = [zs](int i) { return zs[fpad<M>(i)].x; };
    auto fb = [zs](int i) { return -zs[fpad<M>(i)].y; };
    if (L.rowsInterp == kCubic) {
      float4* rr = static_cast<float4*>(L.rows) + rbase;
      for (int j = threadIdx.x; j < rp; j += blockDim.x) {
        rr[j] = interval_elem<kCubic>(fa, j - kRowPad, n);
        if (two) rr[rp + j] = interval_elem<kCubic>(fb, j - kRowPad, n);
      }
    } else if (L.rowsInterp == kLinear) {
      float2* rr = static_cast<float2*>(L.rows) + rbase;
      for (int j = threadIdx.x; j < rp; j += blockDim.x) {
        rr[j] = interval_elem<kLinear>(fa, j - kRowPad, n);
        if (two) rr[rp + j] = interval_elem<kLinear>(fb, j - kRowPad, n);
      }
    } else {
      float* rr = static_cast<float*>(L.rows) + rbase;
      for (int j = threadIdx.x; j < rp; j += blockDim.x) {
        rr[j] = interval_elem<kNearest>(fa, j - kRowPad, n);
        if (two) rr[rp + j] = interval_elem<kNearest>(fb, j - kRowPad, n);
      }
    }
  }
}


// ---------------------------------------------------------------------------
// Persistent variant for batched launches: N = 2^LOG2N fixed at compile time,
// N/16 threads per transform (radix-16 passes, then one radix-8/4/2 pass), and
// each block loops over view pairs.  The sequence lives in shared memory with
// one pad slot after every 16 elements (element m at m + m/16): every pass's
// reads and writes are then free of bank conflicts, and every access is a
// compile-time offset from one per-thread base address.  Each thread's
// twiddle factors for every pass are loaded once into registers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int pslot(int m) { return m + (m >> 4); }

template <int N, int P>
struct PassInfo {
  static constexpr int R = (P * 16 <= N) ? 16 : (P * 8 <= N) ? 8 : (P * 4 == N) ? 4 : 2;
  static constexpr int S = 16 / R;                    // butterflies per thread
  static constexpr int NTW = P > 1 ? S * (R - 1) : 0;  // twiddles per thread
  static constexpr int TOTAL = NTW + PassInfo<N, P * R>::TOTAL;
};
template <int N>
struct PassInfo<N, N> {
  static constexpr int R = 1, S = 0, NTW = 0, TOTAL = 0;
};

template <int N, int P, int OFF, int NT>
__device__ __forceinline__ void load_pass_twiddles(float2 (&twr)[NT], const float2* __restrict__ tw) {
  if constexpr (P < N) {
    using PI = PassInfo<N, P>;
    constexpr int R = PI::R, S = PI::S, T = N / 16, stride = N / (P * R);
    if constexpr (P > 1) {
#pragma unroll
      for (int s = 0; s < S; s++) {
        const int k = (threadIdx.x + s * T) & (P - 1);
#pragma unroll
        for (int r = 1; r < R; r++) twr[OFF + s * (R - 1) + r - 1] = __ldg(&tw[r * k * stride]);
      }
    }
    load_pass_twiddles<N, P * R, OFF + PI::NTW>(twr, tw);
  }
}

template <int N, int P, int OFF, int NT>
__device__ __forceinline__ void run_passes(float2* buf, const float2 (&twr)[NT]) {
  if constexpr (P < N) {
    using PI = PassInfo<N, P>;
    constexpr int R = PI::R, S = PI::S, nb = N / R, T = N / 16;
    static_assert(nb % 16 == 0 && T % 16 == 0, "padded layout needs multiples of 16");
    static_assert(P == 1 || P % 16 == 0, "pass stride");
    float2 u[S][R];
#pragma unroll
    for (int s = 0; s < S; s++) {
      const float2* src = buf + pslot(threadIdx.x) + s * (T + T / 16);
#pragma unroll
      for (int r = 0; r < R; r++) {
        float2 v = src[r * (nb + nb / 16)];
        if constexpr (P > 1)
          if (r > 0) v = cmul(v, twr[OFF + s * (R - 1) + r - 1]);
        u[s][r] = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < S; s++) {
      const int i = threadIdx.x + s * T;
      const int k = i & (P - 1);
      dft<R>(u[s]);
      float2* dst = buf + pslot((i - k) * R + k);
#pragma unroll
      for (int r = 0; r < R; r++) {
        constexpr int step = P == 1 ? 1 : P + P / 16;
        dst[dft_out_index<R>(r) * step] = u[s][r];
      }
    }
    __syncthreads();
    run_passes<N, P * R, OFF + PI::NTW>(buf, twr);
  }
}

// 512 / T blocks of T threads: at most 128 registers, which hold the
// twiddles (27-38 complex values) and one butterfly without spilling
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc, unsigned bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                   (unsigned)__cvta_generic_to_shared(sdst)),
               "l"(gsrc), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int LOG2N>
__global__ void __launch_bounds__((1 << LOG2N) / 16, 512 / ((1 << LOG2N) / 16))
    fft_filter_persistent_kernel(FilterLaunch L, int vec) {
  constexpr int N = 1 << LOG2N, T = N / 16, NQ = N / 4 / T;   // quads per thread (4)
  constexpr int NT = PassInfo<N, 1>::TOTAL;
  // a row has n <= N/2 samples, so only a thread's first JP quads can hold
  // samples; with 16-byte rows, each thread copies those quads of the next
  // pair into its own slots of stg while the current pair is transformed
  constexpr int JP = 2;
  constexpr bool PREF = LOG2N <= 11;   // stg fits the 48 KB of static shared memory
  __shared__ __align__(16) float2 zb[N + N / 16];
  __shared__ __align__(16) float4 stg[PREF ? 2 * JP * T : 1];
  float2 twr[NT > 0 ? NT : 1];
  load_pass_twiddles<N, 1, 0>(twr, L.twiddle);
  const int n = L.nDet;
  const int pairs = (L.nViews + 1) / 2;
  const long long units = (long long)pairs * L.nBatch;
  const bool pref = PREF && vec;
  float4 wr[JP];
#pragma unroll
  for (int j = 0; j < JP; j++) {
    const int m = 4 * (threadIdx.x + j * T);
    float t[4];
#pragma unroll
    for (int e = 0; e < 4; e++) t[e] = m + e < n ? __ldg(&L.weights[m + e]) : 0.f;
    wr[j] = make_float4(t[0], t[1], t[2], t[3]);
  }
  auto prefetch = [&](long long uu) {
    const int z = (int)(uu / pairs), pr = (int)(uu - (long long)z * pairs);
    const int v0 = 2 * pr;
    const bool two = v0 + 1 < L.nViews;
    const float* ia = L.in + (size_t)z * L.inSliceStride + (size_t)v0 * L.inPitch;
    const float* ib = ia + L.inPitch;
#pragma unroll
    for (int j = 0; j < JP; j++) {
      const int m = 4 * (threadIdx.x + j * T);
      const int rem = n - m;
      const unsigned bytes = rem >= 4 ? 16u : rem > 0 ? 4u * rem : 0u;
      cp_async16(&stg[j * T + threadIdx.x], bytes ? ia + m : ia, bytes);
      cp_async16(&stg[(JP + j) * T + threadIdx.x], (two && bytes) ? ib + m : ia,
                 two ? bytes : 0u);
    }
    cp_async_commit();
  };
  if (pref && blockIdx.x < units) prefetch(blockIdx.x);
  for (long long u = blockIdx.x; u < units; u += gridDim.x) {
    const int z = (int)(u / pairs), pr = (int)(u - (long long)z * pairs);
    const int v0 = 2 * pr;
    const bool two = v0 + 1 < L.nViews;
    const float* ia = L.in + (size_t)z * L.inSliceStride + (size_t)v0 * L.inPitch;
    const float* ib = two ? ia + L.inPitch : ia;
    if (pref) {
      // this pair's rows from the thread's own slots, weighted; then the
      // next pair's copies go out
      cp_async_wait_all();
#pragma unroll
      for (int j = 0; j < NQ; j++) {
        const int m = 4 * (threadIdx.x + j * T);
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
        if (j < JP) {
          const float4 w = wr[j < JP ? j : 0];
          a = stg[j * T + threadIdx.x];
          b = stg[(JP + j) * T + threadIdx.x];
          a = make_float4(w.x * a.x, w.y * a.y, w.z * a.z, w.w * a.w);
          b = make_float4(w.x * b.x, w.y * b.y, w.z * b.z, w.w * b.w);
        }
        float2* d = zb + pslot(m);
        d[0] = make_float2(a.x, b.x);
        d[1] = make_float2(a.y, b.y);
        d[2] = make_float2(a.z, b.z);
        d[3] = make_float2(a.w, b.w);
      }
      if (u + gridDim.x < units) prefetch(u + gridDim.x);
    } else {
    // weighted rows a (real part) and b (imaginary part), zero padded to N
#pragma unroll
    for (int j = 0; j < NQ; j++) {
      const int m = 4 * (threadIdx.x + j * T);
      float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
      if (m < n) {
        if (vec && m + 3 < n) {
          const float4 w = __ldg(reinterpret_cast<const float4*>(L.weights + m));
          a = __ldg(reinterpret_cast<const float4*>(ia + m));
          b = __ldg(reinterpret_cast<const float4*>(ib + m));
          a = make_float4(w.x * a.x, w.y * a.y, w.z * a.z, w.w * a.w);
          b = make_float4(w.x * b.x, w.y * b.y, w.z * b.z, w.w * b.w);
        } else {
          float ta[4] = {0.f, 0.f, 0.f, 0.f}, tb[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
          for (int e = 0; e < 4; e++)
            if (m + e < n) {
              const float w = __ldg(&L.weights[m + e]);
              ta[e] = w * __ldg(&ia[m + e]);
              tb[e] = w * __ldg(&ib[m + e]);
            }
          a = make_float4(ta[0], ta[1], ta[2], ta[3]);
          b = make_float4(tb[0], tb[1], tb[2], tb[3]);
        }
        if (!two) b = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      float2* d = zb + pslot(m);
      d[0] = make_float2(a.x, b.x);
      d[1] = make_float2(a.y, b.y);
      d[2] = make_float2(a.z, b.z);
      d[3] = make_float2(a.w, b.w);
    }
    }
    __syncthreads();
    run_passes<N, 1, 0>(zb, twr);
    // product with the kernel's spectrum, conjugated (the next forward
    // transform is then the inverse one)
    {
      float2* d = zb + pslot(threadIdx.x);
      const float2* sp = L.spectrum + threadIdx.x;
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const float2 zz = cmul(d[j * (T + T / 16)], __ldg(&sp[j * T]));
        d[j * (T + T / 16)] = make_float2(zz.x, -zz.y);
      }
    }
    __syncthreads();
    run_passes<N, 1, 0>(zb, twr);
    float* oa = L.out + (size_t)z * L.outSliceStride + (size_t)v0 * L.outPitch;
    float* ob = oa + L.outPitch;
    const int outEnd = vec ? L.outPitch : n;   // vector stores also zero the pitch padding
#pragma unroll
    for (int j = 0; j < NQ; j++) {
      const int m = 4 * (threadIdx.x + j * T);
      if (m < outEnd) {
        const float2* d = zb + pslot(m);
        const float2 y0 = d[0], y1 = d[1], y2 = d[2], y3 = d[3];
        if (vec) {
          float4 ra = make_float4(y0.x, y1.x, y2.x, y3.x);
          float4 rb = make_float4(-y0.y, -y1.y, -y2.y, -y3.y);
          if (m + 3 >= n) {
            if (m + 1 >= n) { ra.y = 0.f; rb.y = 0.f; }
            if (m + 2 >= n) { ra.z = 0.f; rb.z = 0.f; }
            ra.w = 0.f; rb.w = 0.f;
            if (m >= n) { ra.x = 0.f; rb.x = 0.f; }
          }
          *reinterpret_cast<float4*>(oa + m) = ra;
          if (two) *reinterpret_cast<float4*>(ob + m) = rb;
        } else {
          const float ya[4] = {y0.x, y1.x, y2.x, y3.x}, yb[4] = {y0.y, y1.y, y2.y, y3.y};
#pragma unroll
          for (int e = 0; e < 4; e++)
            if (m + e < n) {
              oa[m + e] = ya[e];
              if (two) ob[m + e] = -yb[e];
            }
        }
      }
    }
    // the interval rows of both views, for the table-family backprojection
    // that follows (the same elements interval_rows_kernel would write)
    if (L.rows) {
      const int rp = L.rowsPitch;
      const size_t rbase = (size_t)z * L.rowsSliceStride + (size_t)v0 * rp;
      const float2* zs = zb;
      auto fa = [zs](int i) { return zs[pslot(i)].x; };
      auto fb = [zs](int i) { return -zs[pslot(i)].y; };
      if (L.rowsInterp == kCubic) {
        float4* rr = static_cast<float4*>(L.rows) + rbase;
        for (int j = threadIdx.x; j < rp; j += T) {
          rr[j] = interval_elem<kCubic>(fa, j - kRowPad, n);
          if (two) rr[rp + j] = interval_elem<kCubic>(fb, j - kRowPad, n);
        }
      } else if (L.rowsInterp == kLinear) {
        float2* rr = static_cast<float2*>(L.rows) + rbase;
        for (int j = threadIdx.x; j < rp; j += T) {
          rr[j] = interval_elem<kLinear>(fa, j - kRowPad, n);
          if (two) rr[rp + j] = interval_elem<kLinear>(fb, j - kRowPad, n);
        }
      } else {
        float* rr = static_cast<float*>(L.rows) + rbase;
        for (int j = threadIdx.x; j < rp; j += T) {
          rr[j] = interval_elem<kNearest>(fa, j - kRowPad, n);
          if (two) rr[rp + j] = interval_elem<kNearest>(fb, j - kRowPad, n);
        }
      }
    }
    __syncthreads();   // zb is rewritten by the next pair
  }
}

template <int LOG2N>
static cudaError_t launch_persistent(const FilterLaunch& L, cudaStream_t s, bool* rowsWritten) {
  constexpr int T = (1 << LOG2N) / 16;
  auto kern = fft_filter_persistent_kernel<LOG2N>;
  // resident blocks of this kernel on the device, queried once (thread-safe
  // initialisation; 0 if the query failed)
  static const long long resident = [] {
    int dev = 0, sms = 0, perSm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, fft_filter_persistent_kernel<LOG2N>,
                                                      (1 << LOG2N) / 16, 0) != cudaSuccess)
      return 0LL;
    return (long long)sms * perSm;
  }();
  if (resident < 1) return cudaErrorInvalidValue;
  const long long units = (long long)((L.nViews + 1) / 2) * (L.nBatch > 0 ? L.nBatch : 1);
  const long long grid = std::min<long long>(units, resident);
  const int vec = ((reinterpret_cast<uintptr_t>(L.in) | reinterpret_cast<uintptr_t>(L.out) |
                    reinterpret_cast<uintptr_t>(L.weights)) & 15) == 0 &&
                  (L.inPitch & 3) == 0 && (L.outPitch & 3) == 0 && (L.inSliceStride & 3) == 0 &&
                  (L.outSliceStride & 3) == 0;
  FilterLaunch Lk = L;
  if (Lk.nBatch < 1) Lk.nBatch = 1;
  kern<<<(unsigned)grid, T, 0, s>>>(Lk, vec);
  if (rowsWritten) *rowsWritten = L.rows != nullptr;
  return cudaGetLastError();
}

cudaError_t launch_filter(const FilterLaunch& L, cudaStream_t s, bool* rowsWritten) {
  if (rowsWritten) *rowsWritten = false;
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
  if (!one) {
    switch (N) {
      case 512: return launch_persistent<9>(L, s, rowsWritten);
      case 1024: return launch_persistent<10>(L, s, rowsWritten);
      case 2048: return launch_persistent<11>(L, s, rowsWritten);
      case 4096: return launch_persistent<12>(L, s, rowsWritten);
      default: break;
    }
  }
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
  if (rowsWritten) *rowsWritten = L.rows != nullptr;
  return cudaGetLastError();
}

}  // namespace ctgpu
