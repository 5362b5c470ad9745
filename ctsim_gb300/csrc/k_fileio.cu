// k_fileio.cu -- device side of CTSim's file formats and image utilities on sm_103a.
//
// .pj view records (libctsim/projections.cpp:811-889, detarrayRead /
// detarrayWrite): f64 view angle, u32 nDet, nDet x f32, little-endian, back
// to back after the header.  A record is 3 + nDet 32-bit words, so records
// start on 4-byte boundaries only: the kernels move 32-bit words and build
// the angle from two of them.  Both machines this library targets are
// little-endian, like the files.
//
// pj2if (tools/pj2if.cpp:118-125): image (nDet x nView) with
// v[ix][iy] = view (nView - 1 - iy), detector ix -- a transpose with the views
// reversed, through 64 x 64 shared-memory tiles so that both sides move
// 256-byte runs.
//
// ImageFile::comparativeStatistics (libctsim/imagefile.cpp:186-240), the
// numbers `if2 --comp` prints: d = sqrt(sum (a-b)^2 / sum (a-mean)^2),
// r = sum |a-b| / sum |a|, e = the largest |difference| of 2x2 block means.
// The reference forms a - b and the 2x2 sums in FP32 and sums in FP64.  FP64
// runs at 1/64 of the FP32 rate on this GPU, so per pixel the sums are kept
// as unevaluated pairs of floats (hi + lo, Knuth's two-sum and an FMA for the
// exact square) and only each thread's partials go to FP64, summed in a
// fixed order: the result does not depend on timing, and agrees with the
// reference's sequential FP64 sums to ~1e-12 relative.  One pass over the
// pixels: the squares about the mean are taken about a shift c and corrected
// by the exact identity
// sum (a-m)^2 = sum (a-c)^2 - 2 (m-c) sum (a-c) + n (m-c)^2 at the end; c is
// the mean of 32 evenly spaced pixels, computed alike by every block.
// e is exact: the 2x2 block sums are the reference's FP32 sums, their
// difference is kept exactly as a float pair and the pairs' maximum is
// found by an exact comparison; 0.25 (hi + lo) in FP64 is then the
// reference's FP64 value.  The pixel pass has no FP64 instruction (an FP64
// warp instruction costs as much with one lane active as with 32).
#include "ctgpu_internal.h"

namespace ctgpu {

namespace {

constexpr int kIoThreads = 256;

// ---------------------------------------------------------------- .pj words
// The records of all views are one flat word array; each thread moves four
// consecutive words (one 16-byte store or load on the record side when the
// record array is 16-byte aligned, VEC) and finds their (view, word) by
// division.  IDX is uint32_t while the array has fewer than 2^32 words.
template <class IDX, bool VEC>
__global__ void __launch_bounds__(kIoThreads) pj_pack_kernel(const float* __restrict__ sino,
                                                              int pitch,
                                                              const double* __restrict__ angles,
                                                              int nViews, int nDet,
                                                              uint32_t* __restrict__ out) {
  const IDX rec = 3 + (IDX)nDet, total = rec * (IDX)nViews;
  const IDX quads = (total + 3) / 4;
  for (IDX q = blockIdx.x * (IDX)blockDim.x + threadIdx.x; q < quads;
       q += (IDX)gridDim.x * blockDim.x) {
    const IDX w0 = 4 * q;
    IDX v = w0 / rec, j = w0 - v * rec;
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      uint32_t x = 0;
      if (w0 + k < total) {
        if (j >= 3) {
          x = __float_as_uint(sino[(size_t)v * pitch + (j - 3)]);
        } else if (j == 2) {
          x = (uint32_t)nDet;
        } else {
          const unsigned long long a = (unsigned long long)__double_as_longlong(angles[v]);
          x = (uint32_t)(j == 0 ? a : (a >> 32));
        }
      }
      w[k] = x;
      if (++j == rec) { j = 0; v++; }
    }
    if (VEC && w0 + 4 <= total) {
      *reinterpret_cast<uint4*>(out + w0) = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
      for (int k = 0; k < 4 && w0 + k < total; k++) out[w0 + k] = w[k];
    }
  }
}

// inverse of pj_pack_kernel, one word per thread and step so that loads and
// stores stay coalesced; (view, word) advance by the grid stride.  A record
// whose nDet word differs from the header's raises status[0] (count) and
// lowers status[1] (first such view); pad columns [nDet, pitch) are zeroed.
template <class IDX>
__global__ void __launch_bounds__(kIoThreads) pj_unpack_kernel(const uint32_t* __restrict__ in,
                                                                int nViews, int nDet,
                                                                float* __restrict__ sino,
                                                                int pitch,
                                                                double* __restrict__ angles,
                                                                int viewOffset,
                                                                unsigned int* status) {
  const IDX rec = 3 + (IDX)nDet, total = rec * (IDX)nViews;
  const IDX stride = (IDX)gridDim.x * blockDim.x;
  const IDX sv = stride / rec, sj = stride - sv * rec;
  IDX w = blockIdx.x * (IDX)blockDim.x + threadIdx.x;
  IDX v = w / rec, j = w - v * rec;
  // four words per step, their loads issued together
  for (; w < total; w += 4 * stride) {
    uint32_t x[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const IDX wk = w + (IDX)k * stride;
      x[k] = wk < total ? in[wk] : 0u;
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const IDX wk = w + (IDX)k * stride;
      if (wk < total) {
        if (j >= 3) {
          sino[(size_t)v * pitch + (j - 3)] = __uint_as_float(x[k]);
        } else if (j == 2) {
          if (x[k] != (uint32_t)nDet) {
            atomicAdd(&status[0], 1u);
            atomicMin(&status[1], (unsigned int)(viewOffset + (int)v));
          }
        } else if (j == 1) {
          angles[v] = __hiloint2double((int)x[k], (int)in[wk - 1]);
        }
      }
      v += sv;
      j += sj;
      if (j >= rec) {
        j -= rec;
        v++;
      }
    }
  }
  const IDX padw = (IDX)(pitch - nDet), pads = padw * (IDX)nViews;
  for (IDX p = blockIdx.x * (IDX)blockDim.x + threadIdx.x; p < pads; p += stride) {
    const IDX pv = p / padw, c = p - pv * padw;
    sino[(size_t)pv * pitch + nDet + c] = 0.f;
  }
}

// ------------------------------------------------------------------ pj2if
// 64 x 64 tiles, block (32, 8), 16 elements per thread:
// image[ix][iy] = sino[nView - 1 - iy][ix]
__global__ void __launch_bounds__(256) sino_to_image_kernel(const float* __restrict__ sino,
                                                            int pitch, int nView, int nDet,
                                                            float* __restrict__ image) {
  __shared__ float tile[64][65];
  const int ix0 = blockIdx.x * 64, iy0 = blockIdx.y * 64;
  // read: rows iy (views reversed), detectors ix contiguous
#pragma unroll
  for (int k = threadIdx.y; k < 64; k += 8) {
    const int iy = iy0 + k;
#pragma unroll
    for (int h = 0; h < 64; h += 32) {
      const int ix = ix0 + h + threadIdx.x;
      if (iy < nView && ix < nDet)
        tile[k][h + threadIdx.x] = sino[(size_t)(nView - 1 - iy) * pitch + ix];
    }
  }
  __syncthreads();
  // write: columns ix, rows iy contiguous
#pragma unroll
  for (int k = threadIdx.y; k < 64; k += 8) {
    const int ix = ix0 + k;
#pragma unroll
    for (int h = 0; h < 64; h += 32) {
      const int iy = iy0 + h + threadIdx.x;
      if (ix < nDet && iy < nView) image[(size_t)ix * nView + iy] = tile[h + threadIdx.x][k];
    }
  }
}

// ----------------------------------------------------------- FP64 -> FP32
__global__ void f64_to_f32_kernel(const double* __restrict__ in, float* __restrict__ out,
                                  size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

// ------------------------------------------------------- image arithmetic
// ImageFile::addImages / subtractImages / multiplyImages / divideImages
// (libctsim/imagefile.cpp:378-528) on real images: FP32 operations.  The
// reference's divide tests the array pointer, not the divisor, against 0
// (:519), so it always divides: x / 0 gives inf or nan there and here.
__global__ void image_arith_kernel(int op, const float* __restrict__ a,
                                   const float* __restrict__ b, float* __restrict__ out,
                                   size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float x = a[i], y = b[i];
    float r;
    switch (op) {
      case 0: r = __fadd_rn(x, y); break;
      case 1: r = __fsub_rn(x, y); break;
      case 2: r = __fmul_rn(x, y); break;
      default: r = __fdiv_rn(x, y); break;
    }
    out[i] = r;
  }
}

// ------------------------------------------------- comparative statistics
// s = hi + lo, an unevaluated float pair (~48 significant bits)
struct F2 {
  float hi, lo;
};

// hi + lo = a + b exactly (Knuth's two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float& hi, float& lo) {
  hi = __fadd_rn(a, b);
  const float bb = __fsub_rn(hi, a);
  lo = __fadd_rn(__fsub_rn(a, __fsub_rn(hi, bb)), __fsub_rn(b, bb));
}
// add the exact value x + xl (|xl| <= ulp(x)) to s, renormalised
__device__ __forceinline__ void f2_add(F2& s, float x, float xl) {
  float t, err;
  two_sum(s.hi, x, t, err);
  const float lo = __fadd_rn(err, __fadd_rn(s.lo, xl));
  s.hi = __fadd_rn(t, lo);
  s.lo = __fsub_rn(lo, __fsub_rn(s.hi, t));
}
__device__ __forceinline__ void f2_add(F2& s, float x) {
  float t, err;
  two_sum(s.hi, x, t, err);
  const float lo = __fadd_rn(err, s.lo);
  s.hi = __fadd_rn(t, lo);
  s.lo = __fsub_rn(lo, __fsub_rn(s.hi, t));
}

// |sa - sb| exactly as (h, l) = (|fl(D)|, (D - fl(D)) sign(D)), D = sa - sb;
// pairs order exactly: by h, then l (rounding is monotone).  Initial (-1, 0)
// stands for the reference's eMax = -1.
struct EMax {
  float h, l;
};
__device__ __forceinline__ void emax_take(EMax& m, float h, float l) {
  if (h > m.h || (h == m.h && l > m.l)) {   // nan never raises it, as there
    m.h = h;
    m.l = l;
  }
}

struct CmpAcc {
  F2 sum, sq, ab, dev, av;   // a, (a-b)^2, |a-b|, (a-c)^2, |a|
  EMax e;
};

// one pixel pair; c = the image's shift
__device__ __forceinline__ void cmp_pixel(CmpAcc& q, float a, float b, float c) {
  f2_add(q.sum, a);
  const float d = __fsub_rn(a, b);   // the reference's FP32 a - b
  const float p = __fmul_rn(d, d);
  f2_add(q.sq, p, __fmaf_rn(d, d, -p));
  f2_add(q.ab, fabsf(d));
  // a - c exactly as s + es, then (s + es)^2 ~ s^2 + 2 s es
  float s, es;
  two_sum(a, -c, s, es);
  const float s2 = __fmul_rn(s, s);
  f2_add(q.dev, s2, __fadd_rn(__fmaf_rn(s, s, -s2), 2.f * s * es));
  f2_add(q.av, fabsf(a));
}

// 2x2 block: the reference's FP32 sums v[2i][2j] + v[2i+1][2j] + v[2i][2j+1]
// + v[2i+1][2j+1] (imagefile.cpp:228-229) and the exact difference of the two
__device__ __forceinline__ void cmp_block(CmpAcc& q, float a00, float a10, float a01, float a11,
                                          float b00, float b10, float b01, float b11) {
  const float sa = __fadd_rn(__fadd_rn(__fadd_rn(a00, a10), a01), a11);
  const float sb = __fadd_rn(__fadd_rn(__fadd_rn(b00, b10), b01), b11);
  float s, t;
  two_sum(sa, -sb, s, t);
  if (isinf(s)) t = 0.f;   // an infinite difference: inf, as in FP64
  emax_take(q.e, fabsf(s), s < 0.f ? -t : t);
}

// fixed-order reductions (blockDim 256, 8 warps)
__device__ F2 f2_sum(F2 a, F2 b) {
  F2 r = a;
  f2_add(r, b.hi, b.lo);
  return r;
}
__device__ EMax block_max_e(EMax v, EMax* sh) {
  for (int o = 16; o > 0; o >>= 1)
    emax_take(v, __shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  EMax r = sh[0];
  if (threadIdx.x == 0)
    for (int i = 1; i < (int)(blockDim.x >> 5); i++) emax_take(r, sh[i].h, sh[i].l);
  return r;
}
// the shift c: the FP32 mean of 32 evenly spaced pixels of image a, summed in
// a fixed order (identical in every block of the image)
__device__ __forceinline__ float cmp_shift(const float* a, size_t n) {
  float v = 0.f;
  if (threadIdx.x < 32) {
    v = a[((size_t)threadIdx.x * n) >> 5];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  return v * (1.f / 32.f);
}

// one pass, grid (nb, nImages), FP32 only: partials -> part[img][blk][0..6]
template <bool PAIRS>
__global__ void __launch_bounds__(256) cmp_stats_kernel(CompareLaunch L) {
  __shared__ float shc;
  __shared__ float2 shp[8][6];
  const int img = blockIdx.y;
  const float* a = L.a + (size_t)img * L.strideA;
  const float* b = L.b + (size_t)img * L.strideB;
  const unsigned nx = L.nx, ny = L.ny, hx = nx / 2, hy = ny / 2;
  {
    const float c0 = cmp_shift(a, (size_t)nx * ny);
    if (threadIdx.x == 0) shc = c0;
    __syncthreads();
  }
  const float c = shc;
  CmpAcc q{{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {-1.f, 0.f}};
  const unsigned stride = gridDim.x * blockDim.x;
  const unsigned t0 = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned nq = hx * hy;
  if (t0 < nq) {
    // (column pair, row pair) of block k, advanced by the grid stride without division
    const unsigned sc = stride / hy, sr = stride - sc * hy;
    unsigned ix3 = t0 / hy, iy = t0 - ix3 * hy;
    for (unsigned k = t0; k < nq; k += stride) {
      const size_t o0 = (size_t)(2 * ix3) * ny + 2 * iy, o1 = o0 + ny;
      float a00, a01, a10, a11, b00, b01, b10, b11;
      if (PAIRS) {   // 8-byte aligned pairs (even ny, aligned bases)
        const float2 x0 = *reinterpret_cast<const float2*>(a + o0);
        const float2 x1 = *reinterpret_cast<const float2*>(a + o1);
        const float2 y0 = *reinterpret_cast<const float2*>(b + o0);
        const float2 y1 = *reinterpret_cast<const float2*>(b + o1);
        a00 = x0.x; a01 = x0.y; a10 = x1.x; a11 = x1.y;
        b00 = y0.x; b01 = y0.y; b10 = y1.x; b11 = y1.y;
      } else {
        a00 = a[o0]; a01 = a[o0 + 1]; a10 = a[o1]; a11 = a[o1 + 1];
        b00 = b[o0]; b01 = b[o0 + 1]; b10 = b[o1]; b11 = b[o1 + 1];
      }
      cmp_pixel(q, a00, b00, c);
      cmp_pixel(q, a01, b01, c);
      cmp_pixel(q, a10, b10, c);
      cmp_pixel(q, a11, b11, c);
      cmp_block(q, a00, a10, a01, a11, b00, b10, b01, b11);
      ix3 += sc;
      iy += sr;
      if (iy >= hy) {
        iy -= hy;
        ix3++;
      }
    }
  }
  // pixels outside the 2x2 blocks: row ny-1 of columns < 2 hx (ny odd), column nx-1 (nx odd)
  const unsigned nRow = (ny & 1) ? 2 * hx : 0, nCol = (nx & 1) ? ny : 0;
  for (unsigned k = t0; k < nRow + nCol; k += stride) {
    const size_t o = k < nRow ? (size_t)k * ny + (ny - 1) : (size_t)(nx - 1) * ny + (k - nRow);
    cmp_pixel(q, a[o], b[o], c);
  }
  // warp reductions of the six quantities together, then one barrier
  F2* acc[5] = {&q.sum, &q.sq, &q.ab, &q.dev, &q.av};
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int i = 0; i < 5; i++) {
      F2 u;
      u.hi = __shfl_down_sync(0xffffffffu, acc[i]->hi, o);
      u.lo = __shfl_down_sync(0xffffffffu, acc[i]->lo, o);
      *acc[i] = f2_sum(*acc[i], u);
    }
    emax_take(q.e, __shfl_down_sync(0xffffffffu, q.e.h, o),
              __shfl_down_sync(0xffffffffu, q.e.l, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int i = 0; i < 5; i++) shp[w][i] = make_float2(acc[i]->hi, acc[i]->lo);
    shp[w][5] = make_float2(q.e.h, q.e.l);
  }
  __syncthreads();
  if (threadIdx.x < 6) {   // thread i combines quantity i over the 8 warps
    const int i = threadIdx.x;
    float2* out = L.part + ((size_t)img * gridDim.x + blockIdx.x) * kCmpParts;
    if (i < 5) {
      F2 r{shp[0][i].x, shp[0][i].y};
      for (int k = 1; k < (int)(blockDim.x >> 5); k++) r = f2_sum(r, F2{shp[k][i].x, shp[k][i].y});
      out[i] = make_float2(r.hi, r.lo);
    } else {
      EMax r{shp[0][5].x, shp[0][5].y};
      for (int k = 1; k < (int)(blockDim.x >> 5); k++) emax_take(r, shp[k][5].x, shp[k][5].y);
      out[5] = make_float2(r.h, r.l);
      out[6] = make_float2(c, 0.f);
    }
  }
}

// one block per image, FP64: d, r, e -> out[img][3]
__global__ void __launch_bounds__(256) cmp_final_kernel(CompareLaunch L, int nb) {
  __shared__ double sh[8];
  __shared__ EMax she[8];
  const int img = blockIdx.x;
  const float2* p = L.part + (size_t)img * nb * kCmpParts;
  double s[5];
#pragma unroll
  for (int k = 0; k < 5; k++) {
    double v = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
      const float2 x = p[(size_t)i * kCmpParts + k];
      v += (double)x.x + (double)x.y;
    }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = sh[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); i++) r += sh[i];
    s[k] = r;
  }
  EMax e{-1.f, 0.f};
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    const float2 x = p[(size_t)i * kCmpParts + 5];
    emax_take(e, x.x, x.y);
  }
  e = block_max_e(e, she);
  if (threadIdx.x == 0) {
    const double n = (double)((unsigned int)L.nx * (unsigned int)L.ny);
    const double c = (double)p[6].x, m = s[0] / n, delta = m - c;
    // sum (a - m)^2 = sum (a - c)^2 - 2 (m - c) sum (a - c) + n (m - c)^2
    const double dev = s[3] - 2.0 * delta * (s[0] - n * c) + n * delta * delta;
    L.out[img * 3 + 0] = sqrt(s[1] / dev);
    L.out[img * 3 + 1] = s[2] / s[4];
    // |D| = h + l exactly (48 bits), so 0.25 (h + l) is the reference's
    // fabs(0.25 sa - 0.25 sb) rounded the same way
    L.out[img * 3 + 2] = e.h < 0.f ? -1.0 : 0.25 * ((double)e.h + (double)e.l);
  }
}

unsigned io_blocks(size_t quads) {
  size_t b = (quads + kIoThreads - 1) / kIoThreads;
  const size_t cap = 152 * 8;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

cudaError_t launch_pj_pack(const float* sino, int pitch, const double* angles, int nViews,
                           int nDet, uint32_t* out, cudaStream_t s) {
  if (nViews <= 0) return cudaSuccess;
  const size_t total = (size_t)(3 + nDet) * nViews;
  const unsigned blocks = io_blocks((total + 3) / 4);
  const bool vec = !(reinterpret_cast<uintptr_t>(out) & 15);
  const bool narrow = total + 4 < (1ull << 32);
  if (narrow && vec)
    pj_pack_kernel<uint32_t, true><<<blocks, kIoThreads, 0, s>>>(sino, pitch, angles, nViews, nDet, out);
  else if (narrow)
    pj_pack_kernel<uint32_t, false><<<blocks, kIoThreads, 0, s>>>(sino, pitch, angles, nViews, nDet, out);
  else if (vec)
    pj_pack_kernel<size_t, true><<<blocks, kIoThreads, 0, s>>>(sino, pitch, angles, nViews, nDet, out);
  else
    pj_pack_kernel<size_t, false><<<blocks, kIoThreads, 0, s>>>(sino, pitch, angles, nViews, nDet, out);
  return cudaGetLastError();
}

cudaError_t launch_pj_unpack(const uint32_t* in, int nViews, int nDet, float* sino, int pitch,
                             double* angles, int viewOffset, unsigned int* status,
                             cudaStream_t s) {
  if (nViews <= 0) return cudaSuccess;
  const size_t total = (size_t)(3 + nDet) * nViews;
  const unsigned blocks = io_blocks((total + 3) / 4);
  if (total + (size_t)kIoThreads * 152 * 8 * 4 < (1ull << 32) &&
      (size_t)(pitch - nDet) * nViews < (1ull << 32))
    pj_unpack_kernel<uint32_t><<<blocks, kIoThreads, 0, s>>>(in, nViews, nDet, sino, pitch,
                                                             angles, viewOffset, status);
  else
    pj_unpack_kernel<size_t><<<blocks, kIoThreads, 0, s>>>(in, nViews, nDet, sino, pitch, angles,
                                                           viewOffset, status);
  return cudaGetLastError();
}

cudaError_t launch_sino_to_image(const float* sino, int pitch, int nView, int nDet, float* image,
                                 cudaStream_t s) {
  if (nView <= 0 || nDet <= 0) return cudaSuccess;
  if ((nView + 63) / 64 > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((nDet + 63) / 64, (nView + 63) / 64);
  sino_to_image_kernel<<<grid, dim3(32, 8), 0, s>>>(sino, pitch, nView, nDet, image);
  return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double* in, float* out, size_t n, cudaStream_t s) {
  if (!n) return cudaSuccess;
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  f64_to_f32_kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t launch_image_arith(int op, const float* a, const float* b, float* out, size_t n,
                               cudaStream_t s) {
  if (!n) return cudaSuccess;
  size_t blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  image_arith_kernel<<<(unsigned)blocks, 256, 0, s>>>(op, a, b, out, n);
  return cudaGetLastError();
}

int compare_blocks(int nx, int ny) {
  const size_t nq = (size_t)(nx / 2) * (ny / 2);
  size_t nb = (nq + 256 * 16 - 1) / (256 * 16);   // >= 16 blocks of 2 x 2 per thread
  if (nb < 1) nb = 1;
  if (nb > 128) nb = 128;
  return (int)nb;
}

cudaError_t launch_image_compare(const CompareLaunch& L, cudaStream_t s) {
  if (L.nImages <= 0) return cudaSuccess;
  if (L.nImages > 65535 || (size_t)L.nx * L.ny >= (1ull << 31))
    return cudaErrorInvalidConfiguration;
  const int nb = compare_blocks(L.nx, L.ny);
  dim3 grid(nb, L.nImages);
  const bool pairs = !(L.ny & 1) && !(reinterpret_cast<uintptr_t>(L.a) & 7) &&
                     !(reinterpret_cast<uintptr_t>(L.b) & 7) &&
                     (L.nImages == 1 || (!(L.strideA & 1) && !(L.strideB & 1)));
  if (pairs) cmp_stats_kernel<true><<<grid, 256, 0, s>>>(L);
  else cmp_stats_kernel<false><<<grid, 256, 0, s>>>(L);
  cmp_final_kernel<<<L.nImages, 256, 0, s>>>(L, nb);
  return cudaGetLastError();
}

}  // namespace ctgpu
