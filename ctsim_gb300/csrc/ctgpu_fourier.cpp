// ctgpu_fourier.cpp -- C ABI of the polar and direct-Fourier images
// (declared in include/ctgpu.h): Projections::convertPolar and
// ::convertFFTPolar (libctsim/projections.cpp:953-1180), ImageFile::ifft with
// magnitude and the natural-order shuffle (libctsim/imagefile.cpp:770-826,
// :1175-1198; libctsim/fourier.cpp:31-63), and the two chained as the GUI's
// Fourier reconstruction (src/views.cpp:2828-2849).
//
// The host does what is per image or per geometry: the parallel source rows
// (interpolateToParallel for fan beams, on the device), the pixel centres
// accumulated as calcArrayPolarCoordinates does, the interpolation positions
// of convertFFTPolar and the twiddle tables (FP64).  Scratch is allocated
// stream-ordered and released before the call returns.
#include <cmath>
#include <cstring>
#include <string>
#include <strings.h>
#include <vector>

#include "../../include/ctgpu.h"
#include "ctgpu_internal.h"

using namespace ctgpu;

namespace {

int fail(int code, const std::string& msg) {
  set_last_error(msg.c_str());
  return code;
}
int ok() {
  set_last_error("");
  return CTGPU_OK;
}

#define CUDA_TRY(expr)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (expr);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(CTGPU_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));   \
  } while (0)

// Projections::convertInterpNameToID (projections.cpp:36-50, 90-101): the name
// table holds "nearest" and "bilinear" ("bicubic" is commented out there)
int polar_interp_id(const char* name) {
  if (!name) return -1;
  if (!strcasecmp(name, "nearest")) return 0;
  if (!strcasecmp(name, "bilinear")) return 1;
  return -1;
}

// stream-ordered device scratch, released (and the stream synchronised) on exit
struct Scratch {
  cudaStream_t st;
  std::vector<void*> p;
  explicit Scratch(cudaStream_t s) : st(s) {}
  template <class T>
  cudaError_t get(T*& out, size_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, sizeof(T) * (count ? count : 1), st);
    if (e == cudaSuccess) p.push_back(q);
    out = static_cast<T*>(q);
    return e;
  }
  ~Scratch() {
    for (void* q : p) cudaFreeAsync(q, st);
    cudaStreamSynchronize(st);
  }
};

// exp(-2 pi i m / n), m < n, FP64 -> float2
std::vector<float2> twiddles(int n) {
  std::vector<float2> t(n > 0 ? n : 1);
  for (int m = 0; m < n; m++) {
    const double a = -kTwoPi * m / n;
    t[m] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  return t;
}

// The parallel projections the conversions start from (projections.cpp:
// 963-965): the input itself, or interpolateToParallel of fan-beam data.
struct Source {
  const float* rows;
  int pitch;
  double rotStart, rotInc, detInc;
};
int polar_source(const ctgpu_geometry* g, const float* d_sino, int pitch, const double* h_angles,
                 Scratch& sc, Source* out) {
  if (g->geometry == CTGPU_GEOMETRY_PARALLEL) {
    *out = Source{d_sino, pitch, g->rot_start, g->rot_inc, g->det_inc};
    return CTGPU_OK;
  }
  if (!h_angles) return fail(CTGPU_ERR_INVALID, "fan-beam data needs its view angles");
  const int p2 = (g->n_det + 3) & ~3;
  float* rows = nullptr;
  CUDA_TRY(sc.get(rows, (size_t)g->n_view * p2));
  ctgpu_geometry g2;
  std::vector<double> a2(g->n_view > 0 ? g->n_view : 1);
  int rc = ctgpu_interpolate_to_parallel(g, d_sino, pitch, h_angles, rows, p2, &g2, a2.data(),
                                         (void*)sc.st);
  if (rc != CTGPU_OK) return rc;
  *out = Source{rows, p2, g2.rot_start, g2.rot_inc, g2.det_inc};
  return CTGPU_OK;
}

// pixel centres of calcArrayPolarCoordinates (projections.cpp:1113-1132)
void pixel_centres(int nx, int ny, double viewDiameter, double zeropadRatio,
                   std::vector<double>& xs, std::vector<double>& ys) {
  double xMin = -viewDiameter / 2, xMax = xMin + viewDiameter;
  double yMin = -viewDiameter / 2, yMax = yMin + viewDiameter;
  const double xCent = (xMin + xMax) / 2, yCent = (yMin + yMax) / 2;
  xMin = (xMin - xCent) * zeropadRatio + xCent;
  xMax = (xMax - xCent) * zeropadRatio + xCent;
  yMin = (yMin - yCent) * zeropadRatio + yCent;
  yMax = (yMax - yCent) * zeropadRatio + yCent;
  const double xInc = (xMax - xMin) / nx, yInc = (yMax - yMin) / ny;
  xs.resize(nx);
  ys.resize(ny);
  double x = xMin + xInc / 2;
  for (int ix = 0; ix < nx; x += xInc, ix++) xs[ix] = x;
  double y = yMin + yInc / 2;
  for (int iy = 0; iy < ny; y += yInc, iy++) ys[iy] = y;
}

int check_common(const ctgpu_geometry* g, const float* d_sino, int pitch, int nx, int ny) {
  if (!g || !d_sino) return fail(CTGPU_ERR_INVALID, "null argument");
  if (g->n_view < 1 || g->n_det < 1 || pitch < g->n_det) return fail(CTGPU_ERR_INVALID, "bad sizes");
  if (nx < 1 || ny < 1 || nx > 65535 || ny > 65535) return fail(CTGPU_ERR_INVALID, "bad image size");
  if (g->geometry < 0 || g->geometry > 2) return fail(CTGPU_ERR_INVALID, "Invalid geometry");
  return CTGPU_OK;
}

int polar_run(const Source& src, const ctgpu_geometry* g, int nx, int ny, int interp,
              double zeropadRatio, double detInc, int nPos, const float* data, int complexData,
              int dataPitch, float* d_re, float* d_im, Scratch& sc) {
  std::vector<double> xs, ys;
  pixel_centres(nx, ny, g->view_diameter, zeropadRatio, xs, ys);
  double* d_xy = nullptr;
  CUDA_TRY(sc.get(d_xy, (size_t)nx + ny));
  CUDA_TRY(cudaMemcpyAsync(d_xy, xs.data(), sizeof(double) * nx, cudaMemcpyHostToDevice, sc.st));
  CUDA_TRY(cudaMemcpyAsync(d_xy + nx, ys.data(), sizeof(double) * ny, cudaMemcpyHostToDevice, sc.st));
  PolarLaunch L{};
  L.nx = nx;
  L.ny = ny;
  L.cols = nx < ny ? nx : ny;
  L.xs = d_xy;
  L.ys = d_xy + nx;
  L.rotInc = src.rotInc;
  L.rotStart = src.rotStart;
  L.detInc = detInc;
  L.detCenter = (nPos - 1) / 2.;
  L.data = data;
  L.complexData = complexData;
  L.pitch = dataPitch;
  L.nView = g->n_view;
  L.nPos = nPos;
  L.interp = interp;
  L.outRe = d_re;
  L.outIm = d_im;
  CUDA_TRY(launch_polar(L, sc.st));
  return CTGPU_OK;
}

}  // namespace

extern "C" {

int ctgpu_convert_polar(const ctgpu_geometry* g, const float* d_sino, int pitch,
                        const double* h_view_angles, int nx, int ny, const char* interp_name,
                        float* d_image, void* stream) {
  int rc = check_common(g, d_sino, pitch, nx, ny);
  if (rc != CTGPU_OK) return rc;
  if (!d_image) return fail(CTGPU_ERR_INVALID, "null argument");
  const int interp = polar_interp_id(interp_name);
  if (interp < 0)
    return fail(CTGPU_ERR_INVALID, std::string("Invalid polar interpolation name ") +
                                       (interp_name ? interp_name : "(null)"));
  Scratch sc((cudaStream_t)stream);
  Source src;
  if ((rc = polar_source(g, d_sino, pitch, h_view_angles, sc, &src)) != CTGPU_OK) return rc;
  rc = polar_run(src, g, nx, ny, interp, 1.0, src.detInc, g->n_det, src.rows, 0, src.pitch,
                 d_image, nullptr, sc);
  return rc != CTGPU_OK ? rc : ok();
}

int ctgpu_convert_fft_polar(const ctgpu_geometry* g, const float* d_sino, int pitch,
                            const double* h_view_angles, int nx, int ny, const char* interp_name,
                            int zeropad, float* d_real, float* d_imag, int* n_transform,
                            void* stream) {
  int rc = check_common(g, d_sino, pitch, nx, ny);
  if (rc != CTGPU_OK) return rc;
  if (!d_real || !d_imag) return fail(CTGPU_ERR_INVALID, "null argument");
  const int interp = polar_interp_id(interp_name);
  if (interp < 0)
    return fail(CTGPU_ERR_INVALID, std::string("Invalid polar interpolation name ") +
                                       (interp_name ? interp_name : "(null)"));
  if (zeropad < 0 || zeropad > 8) return fail(CTGPU_ERR_INVALID, "zeropad must be 0..8");
  // projections.cpp:1016-1027
  const unsigned int sq = (unsigned int)nx * (unsigned int)nx + (unsigned int)ny * (unsigned int)ny;
  const int nInterp = (int)(double)std::sqrt((double)sq);
  int N = nInterp;
  if (zeropad > 0) {   // ProcessSignal::addZeropadFactor (procsignal.cpp:867-881)
    const double lb = std::log((double)nInterp) / std::log(2.0);
    N = 1 << ((int)std::floor(lb) + zeropad);
  }
  if (N > 16384 || line_smem_bytes(N) > 200 * 1024)
    return fail(CTGPU_ERR_UNSUPPORTED, "transform length " + std::to_string(N) +
                                           " exceeds the shared-memory transform (16384, or 12800 "
                                           "for lengths other than powers of two)");
  if (n_transform) *n_transform = N;
  Scratch sc((cudaStream_t)stream);
  Source src;
  if ((rc = polar_source(g, d_sino, pitch, h_view_angles, sc, &src)) != CTGPU_OK) return rc;
  const int nDet = g->n_det, nView = g->n_view;
  const double projScale = nInterp / (g->view_diameter * 0.05);
  const double zpRatio = (double)N / (double)nInterp;
  const double interpScale = nDet / (double)nInterp;
  const double fftScale = 1. / (double)(nInterp * nInterp);
  const double dMid = nInterp / 2.;
  std::vector<double> pos(nInterp);
  for (int i = 0; i < nInterp; i++) pos[i] = (nDet / 2.) + (i - dMid) * interpScale;
  const std::vector<float2> tw = twiddles(N);
  double* d_pos = nullptr;
  float2* d_tw = nullptr;
  float2* d_spec = nullptr;
  CUDA_TRY(sc.get(d_pos, nInterp));
  CUDA_TRY(sc.get(d_tw, N));
  CUDA_TRY(sc.get(d_spec, (size_t)nView * N));
  CUDA_TRY(cudaMemcpyAsync(d_pos, pos.data(), sizeof(double) * nInterp, cudaMemcpyHostToDevice, sc.st));
  CUDA_TRY(cudaMemcpyAsync(d_tw, tw.data(), sizeof(float2) * N, cudaMemcpyHostToDevice, sc.st));
  FourierViewsLaunch V{};
  V.sino = src.rows;
  V.pitch = src.pitch;
  V.nView = nView;
  V.nDet = nDet;
  V.nInterp = nInterp;
  V.N = N;
  V.iMid = nInterp / 2;
  V.posTable = d_pos;
  V.projScale = projScale;
  V.fftScale = fftScale;
  V.twiddle = d_tw;
  V.spec = d_spec;
  CUDA_TRY(launch_fourier_views(V, sc.st));
  rc = polar_run(src, g, nx, ny, interp, zpRatio, src.detInc * interpScale, N,
                 reinterpret_cast<const float*>(d_spec), 1, N, d_real, d_imag, sc);
  return rc != CTGPU_OK ? rc : ok();
}

int ctgpu_image_ifft_magnitude(const float* d_real, const float* d_imag, int nx, int ny,
                               float* d_out, void* stream) {
  if (!d_real || !d_imag || !d_out) return fail(CTGPU_ERR_INVALID, "null argument");
  if (nx < 1 || ny < 1) return fail(CTGPU_ERR_INVALID, "bad image size");
  for (int n : {nx, ny})
    if (n > 16384 || line_smem_bytes(n) > 200 * 1024)
      return fail(CTGPU_ERR_UNSUPPORTED, "image side " + std::to_string(n) +
                                             " exceeds the shared-memory transform");
  Scratch sc((cudaStream_t)stream);
  const std::vector<float2> tx = twiddles(nx), ty = twiddles(ny);
  float2 *d_tx = nullptr, *d_ty = nullptr, *d_tmp = nullptr;
  CUDA_TRY(sc.get(d_tx, nx));
  CUDA_TRY(sc.get(d_ty, ny));
  CUDA_TRY(sc.get(d_tmp, (size_t)nx * ny));
  CUDA_TRY(cudaMemcpyAsync(d_tx, tx.data(), sizeof(float2) * nx, cudaMemcpyHostToDevice, sc.st));
  CUDA_TRY(cudaMemcpyAsync(d_ty, ty.data(), sizeof(float2) * ny, cudaMemcpyHostToDevice, sc.st));
  IfftLaunch L{};
  L.nx = nx;
  L.ny = ny;
  L.inRe = d_real;
  L.inIm = d_imag;
  L.tmp = d_tmp;
  L.twX = d_tx;
  L.twY = d_ty;
  L.out = d_out;
  CUDA_TRY(launch_ifft_magnitude(L, sc.st));
  return ok();
}

int ctgpu_reconstruct_fourier(const ctgpu_geometry* g, const float* d_sino, int pitch,
                              const double* h_view_angles, int nx, int ny,
                              const char* interp_name, int zeropad, float* d_image,
                              void* stream) {
  if (!d_image) return fail(CTGPU_ERR_INVALID, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  float* d_c = nullptr;
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d_c), sizeof(float) * 2 * (size_t)nx * ny, st));
  int rc = ctgpu_convert_fft_polar(g, d_sino, pitch, h_view_angles, nx, ny, interp_name, zeropad,
                                   d_c, d_c + (size_t)nx * ny, nullptr, stream);
  if (rc == CTGPU_OK) rc = ctgpu_image_ifft_magnitude(d_c, d_c + (size_t)nx * ny, nx, ny, d_image, stream);
  const std::string msg = rc != CTGPU_OK ? ctgpu_last_error() : "";
  cudaFreeAsync(d_c, st);
  cudaStreamSynchronize(st);
  if (rc != CTGPU_OK) return fail(rc, msg);
  return ok();
}

}  // extern "C"
