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
// reversed, through shared-memory tiles so both sides stay coalesced.
//
// ImageFile::comparativeStatistics (libctsim/imagefile.cpp:186-240), the
// numbers `if2 --comp` prints: d = sqrt(sum (a-b)^2 / sum (a-mean)^2),
// r = sum |a-b| / sum |a|, e = the largest |difference| of 2x2 block means.
// The reference forms a - b and the 2x2 sums in FP32 and sums in FP64.  FP64
// runs at 1/64 of the FP32 rate on this GPU, so per pixel the sums are kept
// as unevaluated pairs of floats (hi + lo, Knuth's two-sum and an FMA for the
// exact square) and only each thread's partials go to FP64, summed in a
// fixed order: the result does not depend on timing, and agrees with the
// reference's sequential FP64 sums to ~1e-12 relative.  e is exact: the 2x2
// block means are the reference's FP32 sums, their difference and maximum
// are taken in FP64.
#include "ctgpu_internal.h"

namespace ctgpu {

namespace {

constexpr int kIoThreads = 256;
constexpr int kIoWords = 4;   // words per thread per record pass

// ---------------------------------------------------------------- .pj words
// grid (ceil((3 + nDet) / (256 * 4)), min(nViews, 65535)); blocks stride over views
__global__ void __launch_bounds__(kIoThreads) pj_pack_kernel(const float* __restrict__ sino,
                                                              int pitch,
                                                              const double* __restrict__ angles,
                                                              int nViews, int nDet,
                                                              uint32_t* __restrict__ out) {
  const int rec = 3 + nDet;
  for (int v = blockIdx.y; v < nViews; v += gridDim.y) {
    const float* row = sino + (size_t)v * pitch;
    uint32_t* o = out + (size_t)v * rec;
    const int base = blockIdx.x * kIoThreads * kIoWords + threadIdx.x;
#pragma unroll
    for (int k = 0; k < kIoWords; k++) {
      const int j = base + k * kIoThreads;
      if (j >= rec) break;
      uint32_t w;
      if (j >= 3) {
        w = __float_as_uint(row[j - 3]);
      } else if (j == 2) {
        w = (uint32_t)nDet;
      } else {
        const long long a = __double_as_longlong(angles[v]);
        w = (uint32_t)(j == 0 ? a : (a >> 32));
      }
      o[j] = w;
    }
  }
}

// inverse of pj_pack_kernel; a record whose nDet word differs from the
// header's raises status[0] (count) and lowers status[1] (first such view);
// pad columns [nDet, pitch) of each row are zeroed
__global__ void __launch_bounds__(kIoThreads) pj_unpack_kernel(const uint32_t* __restrict__ in,
                                                                int nViews, int nDet,
                                                                float* __restrict__ sino,
                                                                int pitch,
                                                                double* __restrict__ angles,
                                                                int viewOffset,
                                                                unsigned int* status) {
  const int rec = 3 + nDet;
  const int span = (pitch > nDet ? 3 + pitch : rec);
  for (int v = blockIdx.y; v < nViews; v += gridDim.y) {
    const uint32_t* r = in + (size_t)v * rec;
    float* row = sino + (size_t)v * pitch;
    const int base = blockIdx.x * kIoThreads * kIoWords + threadIdx.x;
#pragma unroll
    for (int k = 0; k < kIoWords; k++) {
      const int j = base + k * kIoThreads;
      if (j >= span) break;
      if (j >= rec) {
        row[j - 3] = 0.f;
      } else if (j >= 3) {
        row[j - 3] = __uint_as_float(r[j]);
      } else if (j == 2) {
        if (r[2] != (uint32_t)nDet) {
          atomicAdd(&status[0], 1u);
          atomicMin(&status[1], (unsigned int)(viewOffset + v));
        }
      } else if (j == 0) {
        angles[v] = __hiloint2double((int)r[1], (int)r[0]);
      }
    }
  }
}

// ------------------------------------------------------------------ pj2if
// 32 x 32 tiles, block (32, 8): image[ix][iy] = sino[nView - 1 - iy][ix]
__global__ void __launch_bounds__(256) sino_to_image_kernel(const float* __restrict__ sino,
                                                            int pitch, int nView, int nDet,
                                                            float* __restrict__ image) {
  __shared__ float tile[32][33];
  const int ix0 = blockIdx.x * 32, iy0 = blockIdx.y * 32;
  // read: rows iy (views reversed), detectors ix contiguous
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int iy = iy0 + k, ix = ix0 + threadIdx.x;
    if (iy < nView && ix < nDet) tile[k][threadIdx.x] = sino[(size_t)(nView - 1 - iy) * pitch + ix];
  }
  __syncthreads();
  // write: columns ix, rows iy contiguous
  for (int k = threadIdx.y; k < 32; k += 8) {
    const int ix = ix0 + k, iy = iy0 + threadIdx.x;
    if (ix < nDet && iy < nView) image[(size_t)ix * nView + iy] = tile[threadIdx.x][k];
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

// add the exact value x + xl (|xl| <= ulp(x)) to s (Knuth's two-sum, then renormalise)
__device__ __forceinline__ void f2_add(F2& s, float x, float xl) {
  const float t = __fadd_rn(s.hi, x);
  const float bb = __fsub_rn(t, s.hi);
  const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, bb)), __fsub_rn(x, bb));
  const float lo = __fadd_rn(err, __fadd_rn(s.lo, xl));
  s.hi = __fadd_rn(t, lo);
  s.lo = __fsub_rn(lo, __fsub_rn(s.hi, t));
}
__device__ __forceinline__ double f2_value(const F2& s) { return (double)s.hi + (double)s.lo; }

struct CmpAcc {
  F2 sq, ab, dev, av;   // (a-b)^2, |a-b|, (a-c)^2, |a|
  double emax;
};

// one pixel pair; c = (float)mean
__device__ __forceinline__ void cmp_pixel(CmpAcc& q, float a, float b, float c) {
  const float d = __fsub_rn(a, b);
  const float p = __fmul_rn(d, d);
  f2_add(q.sq, p, __fmaf_rn(d, d, -p));
  f2_add(q.ab, fabsf(d), 0.f);
  // a - c exactly as s + es (two-difference), then (s + es)^2 ~ s^2 + 2 s es
  const float s = __fsub_rn(a, c);
  const float bb = __fsub_rn(s, a);
  const float es = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(-c, bb));
  const float s2 = __fmul_rn(s, s);
  f2_add(q.dev, s2, __fmaf_rn(s, s, -s2) + 2.f * s * es);
  f2_add(q.av, fabsf(a), 0.f);
}

// fixed-order block sum of doubles (blockDim 256); result valid in thread 0
__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) r += sh[i];
  return r;
}
__device__ double block_max(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = -1.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) r = fmax(r, sh[i]);
  return r;
}

// pass 1, grid (nb, nImages): partial sums of a -> part[img][blk][0]
__global__ void __launch_bounds__(256) cmp_sum_kernel(CompareLaunch L) {
  const float* a = L.a + (size_t)blockIdx.y * L.strideA;
  const size_t n = (size_t)L.nx * L.ny;
  F2 s{0.f, 0.f};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    f2_add(s, a[i], 0.f);
  __shared__ double sh[32];
  const double t = block_sum(f2_value(s), sh);
  if (threadIdx.x == 0) L.part[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * kCmpParts] = t;
}

// the image's mean from its pass-1 partials, in the same order in every block
__device__ double cmp_mean(const CompareLaunch& L, int img, int nb, double* sh) {
  __shared__ double mean;
  double v = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x)
    v += L.part[((size_t)img * nb + i) * kCmpParts];
  const double t = block_sum(v, sh);
  if (threadIdx.x == 0) mean = t / (double)((unsigned int)L.nx * (unsigned int)L.ny);
  __syncthreads();
  return mean;
}

// pass 2, grid (nb, nImages): the four sums and the 2x2 maximum -> part[img][blk][1..5]
__global__ void __launch_bounds__(256) cmp_stats_kernel(CompareLaunch L) {
  __shared__ double sh[32];
  const int img = blockIdx.y, nb = gridDim.x;
  const double mean = cmp_mean(L, img, nb, sh);
  const float c = (float)mean;
  const float* a = L.a + (size_t)img * L.strideA;
  const float* b = L.b + (size_t)img * L.strideB;
  const int nx = L.nx, ny = L.ny, hx = nx / 2, hy = ny / 2;
  CmpAcc q{{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, -1.0};
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  // 2x2 blocks: columns 2 ix3, 2 ix3 + 1, rows 2 iy, 2 iy + 1 (8-byte aligned pairs)
  const size_t nq = (size_t)hx * hy;
  for (size_t k = t0; k < nq; k += stride) {
    const int ix3 = (int)(k / (size_t)hy), iy = (int)(k - (size_t)ix3 * hy);
    const size_t o0 = (size_t)(2 * ix3) * ny + 2 * iy, o1 = o0 + ny;
    const float a00 = a[o0], a01 = a[o0 + 1], a10 = a[o1], a11 = a[o1 + 1];
    const float b00 = b[o0], b01 = b[o0 + 1], b10 = b[o1], b11 = b[o1 + 1];
    cmp_pixel(q, a00, b00, c);
    cmp_pixel(q, a01, b01, c);
    cmp_pixel(q, a10, b10, c);
    cmp_pixel(q, a11, b11, c);
    // imagefile.cpp:228-229: v[2i][2j] + v[2i+1][2j] + v[2i][2j+1] + v[2i+1][2j+1] in FP32
    const float sa = __fadd_rn(__fadd_rn(__fadd_rn(a00, a10), a01), a11);
    const float sb = __fadd_rn(__fadd_rn(__fadd_rn(b00, b10), b01), b11);
    q.emax = fmax(q.emax, fabs(0.25 * (double)sa - 0.25 * (double)sb));
  }
  // pixels outside the 2x2 blocks: row ny-1 of columns < 2 hx (ny odd), column nx-1 (nx odd)
  const size_t nRow = (ny & 1) ? (size_t)2 * hx : 0, nCol = (nx & 1) ? (size_t)ny : 0;
  for (size_t k = t0; k < nRow + nCol; k += stride) {
    const size_t o = k < nRow ? k * ny + (ny - 1) : (size_t)(nx - 1) * ny + (k - nRow);
    cmp_pixel(q, a[o], b[o], c);
  }
  double* out = L.part + ((size_t)img * nb + blockIdx.x) * kCmpParts;
  double t;
  t = block_sum(f2_value(q.sq), sh);
  if (threadIdx.x == 0) out[1] = t;
  t = block_sum(f2_value(q.ab), sh);
  if (threadIdx.x == 0) out[2] = t;
  t = block_sum(f2_value(q.dev), sh);
  if (threadIdx.x == 0) out[3] = t;
  t = block_sum(f2_value(q.av), sh);
  if (threadIdx.x == 0) out[4] = t;
  t = block_max(q.emax, sh);
  if (threadIdx.x == 0) out[5] = t;
}

// pass 3, one block per image: d, r, e -> out[img][3]
__global__ void __launch_bounds__(256) cmp_final_kernel(CompareLaunch L, int nb) {
  __shared__ double sh[32];
  const int img = blockIdx.x;
  const double* p = L.part + (size_t)img * nb * kCmpParts;
  double acc[5];
  for (int k = 0; k < 5; k++) {
    double v = k == 4 ? -1.0 : 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
      v = k == 4 ? fmax(v, p[(size_t)i * kCmpParts + 5]) : v + p[(size_t)i * kCmpParts + 1 + k];
    acc[k] = k == 4 ? block_max(v, sh) : block_sum(v, sh);
  }
  double s0 = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s0 += p[(size_t)i * kCmpParts];
  s0 = block_sum(s0, sh);
  if (threadIdx.x == 0) {
    const double n = (double)((unsigned int)L.nx * (unsigned int)L.ny);
    const double mean = s0 / n;
    const double c = (double)(float)mean, delta = mean - c;
    // sum (a - mean)^2 = sum (a - c)^2 - 2 delta sum (a - c) + n delta^2
    const double dev = acc[2] - 2.0 * delta * (s0 - n * c) + n * delta * delta;
    L.out[img * 3 + 0] = sqrt(acc[0] / dev);
    L.out[img * 3 + 1] = acc[1] / acc[3];
    L.out[img * 3 + 2] = acc[4];
  }
}

int io_grid_x(int nDet, int pitch) {
  const int span = 3 + (pitch > nDet ? pitch : nDet);
  return (span + kIoThreads * kIoWords - 1) / (kIoThreads * kIoWords);
}

}  // namespace

cudaError_t launch_pj_pack(const float* sino, int pitch, const double* angles, int nViews,
                           int nDet, uint32_t* out, cudaStream_t s) {
  if (nViews <= 0) return cudaSuccess;
  dim3 grid(io_grid_x(nDet, nDet), nViews < 65535 ? nViews : 65535);
  pj_pack_kernel<<<grid, kIoThreads, 0, s>>>(sino, pitch, angles, nViews, nDet, out);
  return cudaGetLastError();
}

cudaError_t launch_pj_unpack(const uint32_t* in, int nViews, int nDet, float* sino, int pitch,
                             double* angles, int viewOffset, unsigned int* status,
                             cudaStream_t s) {
  if (nViews <= 0) return cudaSuccess;
  dim3 grid(io_grid_x(nDet, pitch), nViews < 65535 ? nViews : 65535);
  pj_unpack_kernel<<<grid, kIoThreads, 0, s>>>(in, nViews, nDet, sino, pitch, angles,
                                                viewOffset, status);
  return cudaGetLastError();
}

cudaError_t launch_sino_to_image(const float* sino, int pitch, int nView, int nDet, float* image,
                                 cudaStream_t s) {
  if (nView <= 0 || nDet <= 0) return cudaSuccess;
  if ((nView + 31) / 32 > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid((nDet + 31) / 32, (nView + 31) / 32);
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
  const size_t n = (size_t)nx * ny;
  size_t nb = (n + 256 * 16 - 1) / (256 * 16);
  if (nb < 1) nb = 1;
  if (nb > 128) nb = 128;
  return (int)nb;
}

cudaError_t launch_image_compare(const CompareLaunch& L, cudaStream_t s) {
  if (L.nImages <= 0) return cudaSuccess;
  if (L.nImages > 65535) return cudaErrorInvalidConfiguration;
  const int nb = compare_blocks(L.nx, L.ny);
  dim3 grid(nb, L.nImages);
  cmp_sum_kernel<<<grid, 256, 0, s>>>(L);
  cmp_stats_kernel<<<grid, 256, 0, s>>>(L);
  cmp_final_kernel<<<L.nImages, 256, 0, s>>>(L, nb);
  return cudaGetLastError();
}

}  // namespace ctgpu
