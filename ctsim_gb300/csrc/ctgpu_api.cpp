// ctgpu_api.cpp -- host core and C ABI of libctgpu.so (declared in include/ctgpu.h).
//
// The host side computes everything that is per-object or per-view and cheap,
// in FP64 and in the reference's own order of operations (element transforms
// and outline boxes, scanner geometry, the incrementally rotated view end
// points, filter design, fixed-point backprojection steps), and launches the
// sm_103a kernels for everything that is per ray, per detector sample or per
// pixel.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>
#include <cstring>
#include <string>
#include <strings.h>
#include <vector>

#include "../../include/ctgpu.h"
#include "ctgpu_internal.h"
#include "filter_design.h"

using namespace ctgpu;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int ok() {
  g_err.clear();
  return CTGPU_OK;
}

#define CUDA_TRY(expr)                                                              \
  do {                                                                              \
    cudaError_t e_ = (expr);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(CTGPU_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
cudaError_t ensure_device(T*& p, size_t& cap, size_t count) {
  if (count <= cap && p) return cudaSuccess;
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), sizeof(T) * (count ? count : 1));
  if (e == cudaSuccess) cap = count;
  return e;
}

// ---- 2-D row-vector affine maps (libctsupport/xform.cpp:87-148) -----------
struct M3 { double m[3][3]; };
M3 ident() { M3 r{}; r.m[0][0] = r.m[1][1] = r.m[2][2] = 1; return r; }
M3 xlat(double x, double y) { M3 r = ident(); r.m[2][0] = x; r.m[2][1] = y; return r; }
M3 scalem(double sx, double sy) { M3 r = ident(); r.m[0][0] = sx; r.m[1][1] = sy; return r; }
M3 rotm(double t) {
  M3 r = ident();
  double c = std::cos(t), s = std::sin(t);
  r.m[0][0] = c; r.m[0][1] = s; r.m[1][0] = -s; r.m[1][1] = c;
  return r;
}
M3 mul(const M3& a, const M3& b) {
  M3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      r.m[i][j] = 0;
      for (int k = 0; k < 3; k++) r.m[i][j] += a.m[i][k] * b.m[k][j];
    }
  return r;
}
void apply(const M3& m, double& x, double& y) {
  double xt = x * m.m[0][0] + y * m.m[1][0] + m.m[2][0];
  double yt = x * m.m[0][1] + y * m.m[1][1] + m.m[2][1];
  x = xt;
  y = yt;
}

int elem_type(const char* n) {   // libctsim/phantom.cpp:590-607
  if (!strcasecmp(n, "rectangle")) return kRect;
  if (!strcasecmp(n, "triangle")) return kTriangle;
  if (!strcasecmp(n, "ellipse")) return kEllipse;
  if (!strcasecmp(n, "sector")) return kSector;
  if (!strcasecmp(n, "segment")) return kSegment;
  return 0;
}

int circle_points(double theta) {   // phantom.cpp:821-827
  theta = theta <= 0 ? 0 : (theta >= kTwoPi ? kTwoPi : theta);
  return (int)(360 * theta / kTwoPi + 1.5);
}

void arc(std::vector<double>& x, std::vector<double>& y, int at, int pts, double xc, double yc,
         double r, double start, double stop) {   // phantom.cpp:771-793
  double th = (stop - start) / (pts - 1), c = std::cos(th), s = std::sin(th);
  x[at] = r * std::cos(start) + xc;
  y[at] = r * std::sin(start) + yc;
  double xp = x[at] - xc, yp = y[at] - yc;
  for (int i = 1; i < pts; i++) {
    double xn = c * xp - s * yp, yn = s * xp + c * yp;
    x[at + i] = xn + xc;
    y[at + i] = yn + yc;
    xp = xn;
    yp = yn;
  }
}

// PhantomElement: radians, and the bounding box of the outline polygon the
// reference draws (phantom.cpp:554-566, :669-756); rays missing that box are
// rejected before clipping.
PElem make_elem(int type, double cx, double cy, double u, double v, double rotDeg, double atten) {
  PElem e{};
  e.type = type;
  e.cx = cx; e.cy = cy; e.u = u; e.v = v; e.atten = atten;
  e.rot = rotDeg * (kPi / 180.);
  e.cosr = std::cos(e.rot);
  e.sinr = std::sin(e.rot);
  std::vector<double> x, y;
  switch (type) {
    case kRect:
      x = {-u, u, u, -u, -u}; y = {-v, -v, v, v, -v};
      break;
    case kTriangle:
      x = {-u, u, 0.0, -u}; y = {0.0, 0.0, v, 0.0};
      break;
    case kEllipse: {
      int n = circle_points(kTwoPi);
      x.resize(n); y.resize(n);
      arc(x, y, 0, n, 0, 0, 1.0, 0.0, kTwoPi);
      for (int i = 0; i < n; i++) { x[i] *= u; y[i] *= v; }
      break;
    }
    case kSector: {
      double r = std::sqrt(u * u + v * v), th = std::atan(u / v);
      double start = 3.0 * kHalfPi - th, stop = 3.0 * kHalfPi + th;
      int c = circle_points(stop - start);
      x.resize(c + 3); y.resize(c + 3);
      x[0] = 0.0; y[0] = v; x[1] = -u; y[1] = 0.0;
      arc(x, y, 2, c, 0.0, v, r, start, stop);
      x[c + 2] = 0.0; y[c + 2] = v;
      break;
    }
    case kSegment: {
      double r = std::sqrt(u * u + v * v), th = std::atan(u / v);
      double start = 3.0 * kHalfPi - th, stop = 3.0 * kHalfPi + th;
      int c = circle_points(stop - start);
      x.resize(c + 1); y.resize(c + 1);
      arc(x, y, 0, c, 0.0, v, r, start, stop);
      x[c] = -u; y[c] = 0.0;
      break;
    }
  }
  double c = std::cos(e.rot), s = std::sin(e.rot);
  for (size_t i = 0; i < x.size(); i++) {
    double xr = x[i] * c - y[i] * s, yr = x[i] * s + y[i] * c;
    x[i] = xr + cx;
    y[i] = yr + cy;
  }
  e.bx0 = e.bx1 = x[0];
  e.by0 = e.by1 = y[0];
  for (size_t i = 1; i < x.size(); i++) {
    e.bx0 = std::fmin(e.bx0, x[i]); e.bx1 = std::fmax(e.bx1, x[i]);
    e.by0 = std::fmin(e.by0, y[i]); e.by1 = std::fmax(e.by1, y[i]);
  }
  const double hx = 0.5 * (e.bx1 - e.bx0), hy = 0.5 * (e.by1 - e.by0);
  e.dcbx = (float)(0.5 * (e.bx0 + e.bx1) - cx);
  e.dcby = (float)(0.5 * (e.by0 + e.by1) - cy);
  e.hx = (float)hx;
  e.hy = (float)hy;
  e.rbox = (float)(std::sqrt(hx * hx + hy * hy) * (1.0 + 1e-5) + 1e-7);
  // a line this close to the box centre crosses the box for certain: the
  // kernel's FP32 box test margin (1e-5 (hx + hy)) and its rounding stay inside
  e.rin = (float)(std::fmin(hx, hy) - 2e-5 * (hx + hy) - 1e-7);
  set_elem_quadratic(e);
  return e;
}

int geometry_from_name(const char* n) {   // scanner.cpp:35-41, :254-265
  if (!strcasecmp(n, "parallel")) return kParallel;
  if (!strcasecmp(n, "equiangular")) return kEquiangular;
  if (!strcasecmp(n, "equilinear")) return kEquilinear;
  return -1;
}
int interp_from_name(const char* n) {   // backprojectors.cpp:73-96
  if (!strcasecmp(n, "nearest")) return kNearest;
  if (!strcasecmp(n, "linear")) return kLinear;
  if (!strcasecmp(n, "cubic")) return kCubic;
  return -1;
}
int backproj_from_name(const char* n) {   // backprojectors.cpp:34-46
  if (!strcasecmp(n, "trig")) return kTrig;
  if (!strcasecmp(n, "table")) return kTable;
  if (!strcasecmp(n, "diff")) return kDiff;
  if (!strcasecmp(n, "idiff")) return kIDiff;
  return -1;
}

long long nearest_ll(double x) { return x > 0 ? (long long)(x + 0.5) : (long long)(x - 0.5); }

int pitch_for(int nDet) { return (nDet + 3) & ~3; }

}  // namespace

void ctgpu::set_last_error(const char* msg) { g_err = msg; }

// ===========================================================================
struct ctgpu_phantom {
  std::vector<PElem> elems;   // reference list order: last added first
  double xmin = 1E30, xmax = -1E30, ymin = 1E30, ymax = -1E30;
  bool unitPulse = false;
  PElem* d_elems = nullptr;
  size_t d_cap = 0;
  bool dirty = true;

  cudaError_t upload(cudaStream_t s) {
    if (!dirty && d_elems) return cudaSuccess;
    cudaError_t e = ensure_device(d_elems, d_cap, elems.size());
    if (e != cudaSuccess) return e;
    if (!elems.empty())
      e = cudaMemcpyAsync(d_elems, elems.data(), sizeof(PElem) * elems.size(),
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dirty = false;
    return e;
  }
  ~ctgpu_phantom() { if (d_elems) cudaFree(d_elems); }
};

struct ctgpu_scanner {
  int geometry, nDet, nView, offsetView, nSample;
  double rotLen, rotInc, detInc, detLen, detStart;
  double viewDiameter, scanDiameter, focalLength, centerDetectorLength, sourceDetectorLength;
  double fanBeamAngle, xCenter, yCenter, angularDetLen = 0, angularDetInc = 0;
  double xs1, ys1, xs2, ys2, xd1 = 0, yd1 = 0, xd2 = 0, yd2 = 0;
  M3 inc;
  // the views of the last range asked for (viewsFirst = startView +
  // offsetView, viewsCount of them), and whether d_views / d_sdirs hold
  // their ray records: a scanner does not change after create, so both
  // depend on the range alone and are rebuilt only for another range
  std::vector<ViewPos> views;
  int viewsFirst = 0, viewsCount = -1;
  bool deviceViews = false;
  // the views' ray records and parallel directions on the device
  RayView* d_views = nullptr;
  size_t d_views_cap = 0;
  float2* d_sdirs = nullptr;
  size_t d_sdirs_cap = 0;
  float* d_sino = nullptr;
  size_t d_sino_cap = 0;
  // collect_projections_ellipsoids: the ellipsoids' largest cross-sections,
  // the per-view cross-sections, the ellipsoids' z extents
  PElem* d_belems = nullptr;
  size_t d_belems_cap = 0;
  PElem* d_velems = nullptr;
  size_t d_velems_cap = 0;
  double2* d_zc = nullptr;
  size_t d_zc_cap = 0;
  // equiangular: (cos, sin) of t * delta for every ray index t (the same for
  // every view), for the rays' FP64 box decisions; built for arcN rays of
  // step arcDelta
  double2* d_arc = nullptr;
  size_t d_arc_cap = 0;
  // and in FP32 of the half angles, (cos, sin) of t * delta / 2: the rays'
  // directions
  float2* d_half = nullptr;
  size_t d_half_cap = 0;
  int arcN = 0;
  double arcDelta = 0;
  // the batched ray-sum calls' per-call inputs (elements, offsets, launch
  // descriptors) go up as one copy from a page-locked buffer (two, used in
  // turn: the host fills one while the other's copy may still be queued) to
  // one device buffer
  unsigned char* h_stage[2] = {nullptr, nullptr};
  size_t h_stage_cap[2] = {0, 0};
  cudaEvent_t stage_done[2] = {nullptr, nullptr};
  int stage_next = 0;
  unsigned char* d_stage = nullptr;
  size_t d_stage_cap = 0;
  // the ray records and directions of `views`, built on the host for
  // upload_ray_views
  std::vector<RayView> h_rv;
  std::vector<float2> h_dirs;
  ~ctgpu_scanner() {
    for (void* p : {(void*)d_views, (void*)d_sino, (void*)d_belems,
                    (void*)d_sdirs, (void*)d_velems, (void*)d_zc,
                    (void*)d_arc, (void*)d_half, (void*)d_stage})
      if (p) cudaFree(p);
    for (int b = 0; b < 2; b++) {
      if (h_stage[b]) cudaFreeHost(h_stage[b]);
      if (stage_done[b]) cudaEventDestroy(stage_done[b]);
    }
  }
};

struct ctgpu_recon {
  ctgpu_geometry g;
  int nx, ny, interp, bproj, interpFactor;
  int iDetCenter, pitch;
  int sms = 0;   // SMs of the device (single-slice view groups), queried once
  double xMin, xMax, yMin, yMax, xInc, yInc, rotScale, startR, startPhi;
  FilterDesign fd;
  int fftN = 0;
  float* d_spec = nullptr;   // FilterSpectrum::spectrum, then ::twiddle
  float* d_weights = nullptr;
  float* d_filtered = nullptr;
  size_t d_filtered_cap = 0;
  double* d_angles = nullptr;
  size_t d_angles_cap = 0;
  unsigned char* d_views = nullptr;
  size_t d_views_cap = 0;
  unsigned char* d_scratch = nullptr;
  size_t d_scratch_cap = 0;
  float* d_sino = nullptr;   // run_host staging
  size_t d_sino_cap = 0;
  float* d_image = nullptr;
  size_t d_image_cap = 0;
  // run_batch_host: two chunk buffers each, copy / compute streams and events;
  // chunks of odd index run on s_comp2 with their own filtered rows and
  // set-up scratch, so that consecutive chunks overlap on the device
  float* d_bsino = nullptr;
  size_t d_bsino_cap = 0;
  float* d_bimage = nullptr;
  size_t d_bimage_cap = 0;
  float* d_filtered2 = nullptr;
  size_t d_filtered2_cap = 0;
  unsigned char* d_scratch2 = nullptr;
  size_t d_scratch2_cap = 0;
  cudaStream_t s_in = nullptr, s_comp = nullptr, s_out = nullptr, s_comp2 = nullptr;
  // ctgpu_recon_run: the tile records' stream (beside the filter) and events
  cudaStream_t s_side = nullptr;
  cudaEvent_t sideEv[2] = {};
  // the view angles whose (tile, view) records d_scratch holds, while
  // recKeyValid: ctgpu_recon_run builds them only for other angles, and every
  // other writer of d_scratch's records (or a reallocation) clears the key
  std::vector<double> recKey;
  bool recKeyValid = false;
  cudaEvent_t ev[6] = {};   // in_done[2], comp_done[2], out_done[2]
  double* h_angles_pinned = nullptr;   // page-locked copy of the view angles
  size_t h_angles_cap = 0;
  std::vector<int> hostChunks;         // chunk sizes set by the caller (empty: planned)
  mutable std::vector<int> plannedChunks;   // the last plan, for plannedFor slices on plannedDev
  mutable int plannedFor = 0, plannedDev = -1;
  ~ctgpu_recon() {
    if (h_angles_pinned) cudaFreeHost(h_angles_pinned);
    for (void* p : {(void*)d_spec, (void*)d_weights, (void*)d_filtered, (void*)d_angles,
                    (void*)d_views, (void*)d_scratch, (void*)d_sino, (void*)d_image,
                    (void*)d_bsino, (void*)d_bimage, (void*)d_filtered2, (void*)d_scratch2})
      if (p) cudaFree(p);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : sideEv)
      if (e) cudaEventDestroy(e);
    for (cudaStream_t s : {s_in, s_comp, s_out, s_comp2, s_side})
      if (s) cudaStreamDestroy(s);
  }
};

extern "C" {

const char* ctgpu_last_error(void) { return g_err.c_str(); }
int ctgpu_abi_version(void) { return CTGPU_ABI_VERSION; }

int ctgpu_sync(void* stream) {
  CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  CUDA_TRY(cudaGetLastError());
  unsigned int st = 0;
  CUDA_TRY(status_read_and_clear(&st));
  if (st & kStatusTimeout)
    return fail(CTGPU_ERR_TIMEOUT, "a kernel's bounded shared-memory wait expired; output invalid");
  if (st & kStatusFeatherRange)
    return fail(CTGPU_ERR_INVALID, "HalfScanFeather: complementary view outside the half scan");
  return ok();
}

// ---------------------------------------------------------------- phantom --
int ctgpu_phantom_create(ctgpu_phantom** out) {
  if (!out) return fail(CTGPU_ERR_INVALID, "null output pointer");
  *out = new ctgpu_phantom();
  return ok();
}

int ctgpu_phantom_add_element(ctgpu_phantom* p, const char* type, double cx, double cy, double u,
                              double v, double rot_deg, double atten) {
  if (!p || !type) return fail(CTGPU_ERR_INVALID, "null argument");
  int t = elem_type(type);
  if (!t) return fail(CTGPU_ERR_INVALID, std::string("Unknown PhantomElement type ") + type);
  if (!(u > 0) || !(v > 0)) return fail(CTGPU_ERR_INVALID, "element sizes must be positive");
  PElem e = make_elem(t, cx, cy, u, v, rot_deg, atten);
  p->elems.insert(p->elems.begin(), e);   // std::list::push_front (phantom.cpp:247)
  if (p->xmin > e.bx0) p->xmin = e.bx0;
  if (p->xmax < e.bx1) p->xmax = e.bx1;
  if (p->ymin > e.by0) p->ymin = e.by0;
  if (p->ymax < e.by1) p->ymax = e.by1;
  p->dirty = true;
  return ok();
}

int ctgpu_phantom_create_builtin(const char* name, ctgpu_phantom** out) {
  if (!name || !out) return fail(CTGPU_ERR_INVALID, "null argument");
  static const double shepp[11][6] = {   // phantom.cpp:390-404
      {0.0000, 0.0000, 0.6900, 0.9200, 0.0, 1.00},   {0.0000, -0.0184, 0.6624, 0.8740, 0.0, -0.98},
      {0.2200, 0.0000, 0.1100, 0.3100, -18.0, -0.02}, {-0.2200, 0.0000, 0.1600, 0.4100, 18.0, -0.02},
      {0.0000, 0.3500, 0.2100, 0.2500, 0.0, 0.01},    {0.0000, 0.1000, 0.0460, 0.0460, 0.0, 0.01},
      {0.0000, -0.1000, 0.0460, 0.0460, 0.0, 0.01},   {-0.0800, -0.6050, 0.0460, 0.0230, 0.0, 0.01},
      {0.0000, -0.6050, 0.0230, 0.0230, 0.0, 0.01},   {0.0600, -0.6050, 0.0230, 0.0230, 0.0, 0.01},
      {0.5538, -0.3858, 0.0330, 0.2060, -18.0, 0.03}};
  static const struct { const char* t; double a[6]; } herman[15] = {   // phantom.cpp:415-433
      {"ellipse", {0.000, 1.50, 0.375, 0.3000, 90.00, -0.003}},
      {"ellipse", {0.675, -0.75, 0.225, 0.1500, 140.00, 0.010}},
      {"ellipse", {0.750, 1.50, 0.375, 0.2250, 50.00, 0.003}},
      {"segment", {1.375, -7.50, 1.100, 0.6250, 19.20, -0.204}},
      {"segment", {1.375, -7.50, 1.100, 4.3200, 19.21, 0.204}},
      {"segment", {0.000, -2.25, 1.125, 0.3750, 0.00, -0.003}},
      {"segment", {0.000, -2.25, 1.125, 3.0000, 0.00, 0.003}},
      {"segment", {-1.000, 3.75, 1.000, 0.5000, 135.00, -0.003}},
      {"segment", {-1.000, 3.75, 1.000, 3.0000, 135.00, 0.003}},
      {"segment", {1.000, 3.75, 1.000, 0.5000, 225.00, -0.003}},
      {"segment", {1.000, 3.75, 1.000, 3.0000, 225.00, 0.003}},
      {"triangle", {5.025, 3.75, 1.125, 0.5000, 110.75, 0.206}},
      {"triangle", {-5.025, 3.75, 1.125, 0.9000, -110.75, 0.206}},
      {"ellipse", {0.000, 0.00, 8.625, 6.4687, 90.00, 0.416}},
      {"ellipse", {0.000, 0.00, 7.875, 5.7187, 90.00, -0.206}}};
  ctgpu_phantom* p = new ctgpu_phantom();
  if (!strcasecmp(name, "shepp-logan")) {
    for (auto& r : shepp) ctgpu_phantom_add_element(p, "ellipse", r[0], r[1], r[2], r[3], r[4], r[5]);
  } else if (!strcasecmp(name, "herman")) {
    for (auto& r : herman)
      ctgpu_phantom_add_element(p, r.t, r.a[0], r.a[1], r.a[2], r.a[3], r.a[4], r.a[5]);
  } else if (!strcasecmp(name, "unit-pulse")) {
    p->unitPulse = true;
    ctgpu_phantom_add_element(p, "rectangle", 0., 0., 100., 100., 0., 0.);
    ctgpu_phantom_add_element(p, "ellipse", 0., 0., 1., 1., 0., 1.);
  } else {
    delete p;
    return fail(CTGPU_ERR_INVALID, std::string("Invalid phantom name ") + name);
  }
  *out = p;
  return ok();
}

int ctgpu_phantom_read_file(ctgpu_phantom* p, const char* filename) {
  if (!p || !filename) return fail(CTGPU_ERR_INVALID, "null argument");
  FILE* fp = std::fopen(filename, "r");
  if (!fp) return fail(CTGPU_ERR_IO, std::string("cannot open phantom file ") + filename);
  int rc = CTGPU_OK;
  std::string bad;
  while (true) {   // phantom.cpp:195-209
    char type[80];
    double cx, cy, u, v, rot, dens;
    int st = std::fscanf(fp, "%79s %lf %lf %lf %lf %lf %lf", type, &cx, &cy, &u, &v, &rot, &dens);
    if (st == EOF) break;
    if (st != 7) { rc = CTGPU_ERR_INVALID; bad = "Insufficient fields reading phantom file"; break; }
    int r = ctgpu_phantom_add_element(p, type, cx, cy, u, v, rot, dens);
    if (r != CTGPU_OK) { rc = r; bad = g_err; break; }
  }
  std::fclose(fp);
  return rc == CTGPU_OK ? ok() : fail(rc, bad);
}

int ctgpu_phantom_bounds(const ctgpu_phantom* p, double bounds[4], int* n_elements) {
  if (!p) return fail(CTGPU_ERR_INVALID, "null phantom");
  if (bounds) { bounds[0] = p->xmin; bounds[1] = p->xmax; bounds[2] = p->ymin; bounds[3] = p->ymax; }
  if (n_elements) *n_elements = (int)p->elems.size();
  return ok();
}

void ctgpu_phantom_destroy(ctgpu_phantom* p) { delete p; }

// ---------------------------------------------------------------- scanner --
int ctgpu_scanner_create(const ctgpu_phantom* p, const char* geometry_name, int nDet, int nView,
                         int offsetView, int nSample, double rotAngle, double flRatio,
                         double cdRatio, double viewRatio, double scanRatio, ctgpu_scanner** out) {
  if (!p || !geometry_name || !out) return fail(CTGPU_ERR_INVALID, "null argument");
  int geom = geometry_from_name(geometry_name);
  if (geom < 0) return fail(CTGPU_ERR_INVALID, std::string("Invalid geometry name ") + geometry_name);
  if (nView < 1 || nDet < 1) return fail(CTGPU_ERR_INVALID, "nView & nDet must be greater than 0");
  if (nSample < 1) return fail(CTGPU_ERR_INVALID, "nSample must be greater than 0");
  if (p->elems.empty()) return fail(CTGPU_ERR_INVALID, "phantom has no elements");
  ctgpu_scanner* s = new ctgpu_scanner();
  s->geometry = geom; s->nDet = nDet; s->nView = nView; s->offsetView = offsetView;
  s->nSample = nSample;
  // Scanner::Scanner (scanner.cpp:110-222)
  double maxAxis = (p->xmax - p->xmin) > (p->ymax - p->ymin) ? (p->xmax - p->xmin) : (p->ymax - p->ymin);
  s->viewDiameter = kSqrt2 * maxAxis * viewRatio;
  s->focalLength = (s->viewDiameter / 2) * flRatio;
  s->centerDetectorLength = (s->viewDiameter / 2) * cdRatio;
  s->sourceDetectorLength = s->focalLength + s->centerDetectorLength;
  s->scanDiameter = s->viewDiameter * scanRatio;
  s->xCenter = p->xmin + (p->xmax - p->xmin) / 2;
  s->yCenter = p->ymin + (p->ymax - p->ymin) / 2;
  s->rotLen = rotAngle;
  s->rotInc = s->rotLen / nView;
  bool even = (nDet % 2) == 0;
  if (geom == kParallel) {
    s->fanBeamAngle = 0;
    s->detLen = s->scanDiameter;
    s->detStart = -s->detLen / 2;
    s->detInc = s->detLen / nDet;
    double endOff = 0;
    if (even) { s->detInc = s->detLen / (nDet - 1); endOff = s->detInc; }
    double half = s->detLen / 2;
    s->xs1 = s->xCenter - half; s->ys1 = s->yCenter + s->focalLength;
    s->xs2 = s->xCenter + half + endOff; s->ys2 = s->yCenter + s->focalLength;
    s->xd1 = s->xCenter - half; s->yd1 = s->yCenter - s->centerDetectorLength;
    s->xd2 = s->xCenter + half + endOff; s->yd2 = s->yCenter - s->centerDetectorLength;
    s->detLen += endOff;
  } else if (geom == kEquilinear) {
    if (s->scanDiameter / 2 >= s->focalLength) {
      delete s;
      return fail(CTGPU_ERR_INVALID, "Invalid geometry: Focal length must be larger than scan length");
    }
    double ang = std::asin((s->scanDiameter / 2) / s->focalLength);
    double half = s->sourceDetectorLength * std::tan(ang);
    s->detLen = half * 2;
    s->detStart = -half;
    s->detInc = s->detLen / nDet;
    double endOff = 0;
    if (even) { s->detInc = s->detLen / (nDet - 1); endOff = s->detInc; s->detLen += endOff; }
    s->fanBeamAngle = ang * 2;
    s->xs1 = s->xCenter; s->ys1 = s->yCenter + s->focalLength;
    s->xs2 = s->xCenter; s->ys2 = s->yCenter + s->focalLength;
    s->xd1 = s->xCenter - half; s->yd1 = s->yCenter - s->centerDetectorLength;
    s->xd2 = s->xCenter + half + endOff; s->yd2 = s->yCenter - s->centerDetectorLength;
  } else {
    if (s->scanDiameter / 2 > s->focalLength) {
      delete s;
      return fail(CTGPU_ERR_INVALID, "Invalid geometry: Focal length must be larger than scan length");
    }
    double ang = std::asin((s->scanDiameter / 2) / s->focalLength);
    s->detLen = 2 * ang;
    s->detStart = -ang;
    s->detInc = s->detLen / nDet;
    double endOff = 0;
    if (even) { s->detInc = s->detLen / (nDet - 1); endOff = s->detInc; }
    double a1 = std::acos((s->scanDiameter / 2) / s->centerDetectorLength);
    double angScale = 2 * (kHalfPi + ang - a1) / s->detLen;
    s->angularDetLen = angScale * (s->detLen + endOff);
    s->angularDetInc = angScale * s->detInc;
    s->fanBeamAngle = ang * 2;
    s->xs1 = s->xCenter; s->ys1 = s->yCenter + s->focalLength;
    s->xs2 = s->xCenter; s->ys2 = s->yCenter + s->focalLength;
    s->detLen += endOff;
  }
  s->inc = mul(mul(xlat(-s->xCenter, -s->yCenter), rotm(s->rotInc)), xlat(s->xCenter, s->yCenter));
  *out = s;
  return ok();
}

int ctgpu_scanner_geometry(const ctgpu_scanner* s, ctgpu_geometry* g) {
  if (!s || !g) return fail(CTGPU_ERR_INVALID, "null argument");
  std::memset(g, 0, sizeof(*g));   // Projections::initFromScanner (projections.cpp:145-161)
  g->geometry = s->geometry;
  g->n_det = s->nDet;
  g->n_view = s->nView;
  g->rot_start = s->offsetView * s->rotInc;
  g->rot_inc = s->rotInc;
  g->det_start = s->detStart;
  g->det_inc = s->detInc;
  g->view_diameter = s->viewDiameter;
  g->focal_length = s->focalLength;
  g->source_detector_length = s->sourceDetectorLength;
  g->fan_beam_angle = s->fanBeamAngle;
  return ok();
}

void ctgpu_scanner_destroy(ctgpu_scanner* s) { delete s; }

// View end points by the reference's incremental rotation (scanner.cpp:301-417).
static void scanner_views(ctgpu_scanner* s, int startView, int nViews, int offsetView) {
  if (s->viewsCount == nViews && s->viewsFirst == startView + offsetView) return;
  s->viewsFirst = startView + offsetView;
  s->viewsCount = nViews;
  s->deviceViews = false;
  s->views.resize(nViews);
  double start = (startView + offsetView) * s->rotInc;
  M3 m0 = mul(mul(xlat(-s->xCenter, -s->yCenter), rotm(start)), xlat(s->xCenter, s->yCenter));
  double xd1 = 0, yd1 = 0, xd2 = 0, yd2 = 0;
  if (s->geometry != kEquiangular) {
    xd1 = s->xd1; yd1 = s->yd1; xd2 = s->xd2; yd2 = s->yd2;
    apply(m0, xd1, yd1);
    apply(m0, xd2, yd2);
  }
  double xs1 = s->xs1, ys1 = s->ys1, xs2 = s->xs2, ys2 = s->ys2;
  apply(m0, xs1, ys1);
  apply(m0, xs2, ys2);
  double ang = start;
  for (int v = 0; v < nViews; v++, ang += s->rotInc) {
    s->views[v] = ViewPos{xs1, ys1, xs2, ys2, xd1, yd1, xd2, yd2, ang};
    apply(s->inc, xs1, ys1);
    apply(s->inc, xs2, ys2);
    if (s->geometry != kEquiangular) {
      apply(s->inc, xd1, yd1);
      apply(s->inc, xd2, yd2);
    }
  }
}

}  // extern "C"

// Scanner::projectSingleView's per-view ray geometry (scanner.cpp:445-533)
// in FP64, once per view for every phantom.
RayView ctgpu::make_ray_view(int geometry, int nDet, int nS, double angularDetLen,
                             double angularDetInc, const ViewPos& vp) {
  RayView g{};
  const double sdx = (vp.xs2 - vp.xs1) / nDet, sdy = (vp.ys2 - vp.ys1) / nDet;
  g.S0x = vp.xs1 + sdx / 2;
  g.S0y = vp.ys1 + sdy / 2;
  g.dSx = sdx;
  g.dSy = sdy;
  g.c0 = 1.0;
  if (geometry == kEquiangular) {
    g.delta = angularDetInc / nS;
    g.alpha0 = vp.angle + 3 * kHalfPi - (angularDetLen / 2) + g.delta / 2;
    const double mid = g.alpha0 + 0.5 * (nDet * nS - 1) * g.delta;
    g.c0 = std::cos(g.alpha0);
    g.s0 = std::sin(g.alpha0);
    g.cm = std::cos(mid);
    g.sm = std::sin(mid);
    g.midRel = mid - g.alpha0;
    g.invDelta = 1.0 / g.delta;
  } else {
    const double ddx = (vp.xd2 - vp.xd1) / nDet, ddy = (vp.yd2 - vp.yd1) / nDet;
    const double ddx2 = ddx / nS, ddy2 = ddy / nS;
    g.D0x = vp.xd1 + ddx2 / 2;
    g.D0y = vp.yd1 + ddy2 / 2;
    g.dDx = ddx2;
    g.dDy = ddy2;
  }
  g.rsx = (float)(g.D0x - g.S0x);
  g.rsy = (float)(g.D0y - g.S0y);
  g.stx = (float)g.dDx;
  g.sty = (float)g.dDy;
  g.hdelta = (float)(0.5 * g.delta);
  g.ca0 = (float)g.c0;
  g.sa0 = (float)g.s0;
  g.Sx = (float)g.S0x;
  g.Sy = (float)g.S0y;
  g.cmf = (float)g.cm;
  g.smf = (float)g.sm;
  g.midRelf = (float)g.midRel;
  g.invDeltaf = (float)g.invDelta;
  return g;
}

// the scanner's current views as ray records, and for parallel rays their
// directions ([view][sample]), into host memory
static void fill_ray_views(const ctgpu_scanner* s, int nViews, RayView* rv, float2* dirs) {
  for (int v = 0; v < nViews; v++)
    rv[v] = make_ray_view(s->geometry, s->nDet, s->nSample, s->angularDetLen, s->angularDetInc,
                          s->views[v]);
  if (s->geometry != kParallel) return;
  for (int v = 0; v < nViews; v++)
    for (int i = 0; i < s->nSample; i++) {
      const RayView& g = rv[v];
      double drx = (g.D0x + i * g.dDx) - g.S0x, dry = (g.D0y + i * g.dDy) - g.S0y;
      double inv = 1.0 / std::sqrt(drx * drx + dry * dry);
      dirs[(size_t)v * s->nSample + i] = make_float2((float)(drx * inv), (float)(dry * inv));
    }
}

// equiangular: the scanner's tables of (cos, sin) of t * delta and of
// t * delta / 2 (built once)
static cudaError_t ensure_arc_table(ctgpu_scanner* s) {
  if (s->geometry != kEquiangular) return cudaSuccess;
  const int n = s->nDet * s->nSample;
  const double delta = s->angularDetInc / s->nSample;
  if (s->arcN == n && s->arcDelta == delta) return cudaSuccess;
  std::vector<double2> arc(n);
  std::vector<float2> half(n);
  for (int t = 0; t < n; t++) {
    arc[t] = make_double2(std::cos(t * delta), std::sin(t * delta));
    half[t] = make_float2((float)std::cos(0.5 * t * delta), (float)std::sin(0.5 * t * delta));
  }
  cudaError_t e = ensure_device(s->d_arc, s->d_arc_cap, (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_arc, arc.data(), sizeof(double2) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = ensure_device(s->d_half, s->d_half_cap, (size_t)n);
  if (e == cudaSuccess) e = cudaMemcpy(s->d_half, half.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return e;
  s->arcN = n;
  s->arcDelta = delta;
  return cudaSuccess;
}

// the scanner's current views (scanner_views) as ray records (+ parallel ray
// directions) in d_views / d_sdirs, built and uploaded only when the views
// changed since the last upload.  The copies are from pageable memory: the
// stream's earlier work (which may read the old records) finishes first.
static cudaError_t upload_ray_views(ctgpu_scanner* s, cudaStream_t st) {
  cudaError_t e = ensure_arc_table(s);
  if (e != cudaSuccess || s->deviceViews) return e;
  const int nViews = s->viewsCount;
  s->h_rv.resize(nViews);
  s->h_dirs.resize(s->geometry == kParallel ? (size_t)nViews * s->nSample : 0);
  fill_ray_views(s, nViews, s->h_rv.data(), s->h_dirs.data());
  e = ensure_device(s->d_views, s->d_views_cap, (size_t)(nViews > 0 ? nViews : 1));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->d_views, s->h_rv.data(), sizeof(RayView) * nViews,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !s->h_dirs.empty()) {
    e = ensure_device(s->d_sdirs, s->d_sdirs_cap, s->h_dirs.size());
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s->d_sdirs, s->h_dirs.data(), sizeof(float2) * s->h_dirs.size(),
                          cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) s->deviceViews = true;
  return e;
}

// The scanner's page-locked staging buffer (two, used in turn) for `total`
// bytes, after its last copy is done: the host fills it, stage_send sends it
// to s->d_stage in one asynchronous copy on st.  Copies from pageable memory
// block the host and each sits in the stream as its own transfer.
static cudaError_t stage_host(ctgpu_scanner* s, size_t total, unsigned char** h, int* slot) {
  const int b = s->stage_next;
  s->stage_next ^= 1;
  cudaError_t e = s->stage_done[b] ? cudaEventSynchronize(s->stage_done[b])
                                   : cudaEventCreateWithFlags(&s->stage_done[b], cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  if (s->h_stage_cap[b] < total) {
    if (s->h_stage[b]) cudaFreeHost(s->h_stage[b]);
    s->h_stage[b] = nullptr;
    s->h_stage_cap[b] = 0;
    e = cudaHostAlloc(reinterpret_cast<void**>(&s->h_stage[b]), total, cudaHostAllocDefault);
    if (e != cudaSuccess) return e;
    s->h_stage_cap[b] = total;
  }
  *h = s->h_stage[b];
  *slot = b;
  return cudaSuccess;
}
static cudaError_t stage_send(ctgpu_scanner* s, int slot, size_t total, cudaStream_t st) {
  cudaError_t e = ensure_device(s->d_stage, s->d_stage_cap, total);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->d_stage, s->h_stage[slot], total, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaEventRecord(s->stage_done[slot], st);
  return e;
}
static size_t up16(size_t x) { return (x + 15) & ~(size_t)15; }
extern "C" {

int ctgpu_collect_projections(ctgpu_scanner* s, const ctgpu_phantom* p, int startView,
                              int nViews, int offsetView, int storageOffset, float* d_sino,
                              int pitch, double* h_angles, void* stream) {
  if (!s || !p || !d_sino) return fail(CTGPU_ERR_INVALID, "null argument");
  if (pitch < s->nDet) return fail(CTGPU_ERR_INVALID, "sinogram pitch smaller than nDet");
  if (nViews < 0 || storageOffset < 0) return fail(CTGPU_ERR_INVALID, "negative view range");
  if (nViews == 0) return ok();
  cudaStream_t st = (cudaStream_t)stream;
  scanner_views(s, startView, nViews, offsetView);
  if (h_angles)
    for (int v = 0; v < nViews; v++) h_angles[storageOffset + v] = s->views[v].angle;
  if (p->unitPulse) {   // scanner.cpp:475-478
    CUDA_TRY(launch_unit_pulse(d_sino, nViews, s->nDet, pitch, storageOffset, st));
    return ok();
  }
  CUDA_TRY(const_cast<ctgpu_phantom*>(p)->upload(st));
  CUDA_TRY(upload_ray_views(s, st));
  RaysumLaunch L{};
  L.geometry = s->geometry;
  L.nDet = s->nDet;
  L.nSample = s->nSample;
  L.nElem = (int)p->elems.size();
  L.nViews = nViews;
  L.pitch = pitch;
  L.rowOffset = storageOffset;
  L.centerDetectorLength = s->centerDetectorLength;
  L.angularDetLen = s->angularDetLen;
  L.angularDetInc = s->angularDetInc;
  L.elems = p->d_elems;
  L.views = s->d_views;
  L.sdirs = s->geometry == kParallel ? s->d_sdirs : nullptr;
  L.arc = s->d_arc;
  L.arcHalf = s->d_half;
  L.sino = d_sino;
  L.status = status_pointer();
  cudaError_t e = launch_raysum(L, st);
  if (e == cudaErrorInvalidValue)
    return fail(CTGPU_ERR_UNSUPPORTED, "too many phantom elements x rays per detector for one CTA");
  CUDA_TRY(e);
  return ok();
}

int ctgpu_collect_projections_batch(ctgpu_scanner* s, const ctgpu_phantom* const* phantoms,
                                    int n, float* d_sinos, int pitch, long long sliceStride,
                                    double* h_angles, void* stream) {
  if (!s || !phantoms || !d_sinos || n < 1) return fail(CTGPU_ERR_INVALID, "null argument");
  if (pitch < s->nDet) return fail(CTGPU_ERR_INVALID, "sinogram pitch smaller than nDet");
  if (sliceStride < (long long)pitch * s->nView) return fail(CTGPU_ERR_INVALID, "slice stride too small");
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<PElem> all;
  std::vector<int> offs(1, 0);
  int maxElem = 0;
  for (int z = 0; z < n; z++) {
    const ctgpu_phantom* p = phantoms[z];
    if (!p) return fail(CTGPU_ERR_INVALID, "null phantom");
    if (p->unitPulse) return fail(CTGPU_ERR_UNSUPPORTED, "unit-pulse phantoms are not batched");
    all.insert(all.end(), p->elems.begin(), p->elems.end());
    offs.push_back((int)all.size());
    maxElem = std::max(maxElem, (int)p->elems.size());
  }
  scanner_views(s, 0, s->nView, 0);
  if (h_angles)
    for (int v = 0; v < s->nView; v++) h_angles[v] = s->views[v].angle;
  CUDA_TRY(upload_ray_views(s, st));
  // one staging copy: [elements][offsets]
  const size_t oE = 0;
  const size_t oO = up16(oE + sizeof(PElem) * all.size());
  const size_t total = oO + sizeof(int) * offs.size();
  unsigned char* h = nullptr;
  int slot = 0;
  CUDA_TRY(stage_host(s, total, &h, &slot));
  if (!all.empty()) std::memcpy(h + oE, all.data(), sizeof(PElem) * all.size());
  std::memcpy(h + oO, offs.data(), sizeof(int) * offs.size());
  CUDA_TRY(stage_send(s, slot, total, st));
  RaysumLaunch L{};
  L.geometry = s->geometry;
  L.nDet = s->nDet;
  L.nSample = s->nSample;
  L.nElem = maxElem;
  L.nViews = s->nView;
  L.pitch = pitch;
  L.rowOffset = 0;
  L.centerDetectorLength = s->centerDetectorLength;
  L.angularDetLen = s->angularDetLen;
  L.angularDetInc = s->angularDetInc;
  L.elems = reinterpret_cast<const PElem*>(s->d_stage + oE);
  L.views = s->d_views;
  L.sdirs = s->geometry == kParallel ? s->d_sdirs : nullptr;
  L.arc = s->d_arc;
  L.arcHalf = s->d_half;
  L.sino = d_sinos;
  L.status = status_pointer();
  L.nSlices = n;
  L.elemOffset = reinterpret_cast<const int*>(s->d_stage + oO);
  L.sliceStride = (size_t)sliceStride;
  cudaError_t e = launch_raysum(L, st);
  if (e == cudaErrorInvalidValue)
    return fail(CTGPU_ERR_UNSUPPORTED, "too many phantom elements x rays per detector for one CTA");
  CUDA_TRY(e);
  // (copies from pageable host memory are staged before cudaMemcpyAsync
  // returns, so the vectors may go)
  return ok();
}

int ctgpu_collect_projections_multi(ctgpu_scanner* const* scanners,
                                    const ctgpu_phantom* const* phantoms, int n,
                                    float* const* d_sinos, const int* pitches,
                                    double* const* h_angles, void* stream) {
  if (!scanners || !phantoms || !d_sinos || !pitches || n < 1)
    return fail(CTGPU_ERR_INVALID, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  // each scanner's ray records and directions stay on the device
  // (upload_ray_views); one staging copy: per problem its elements, then the
  // problems' launch descriptors and the block-offset table
  std::vector<size_t> oE(n);
  size_t total = 0;
  for (int k = 0; k < n; k++) {
    ctgpu_scanner* s = scanners[k];
    const ctgpu_phantom* p = phantoms[k];
    if (!s || !p || !d_sinos[k]) return fail(CTGPU_ERR_INVALID, "null scanner, phantom or sinogram");
    if (pitches[k] < s->nDet) return fail(CTGPU_ERR_INVALID, "sinogram pitch smaller than nDet");
    if (p->unitPulse) return fail(CTGPU_ERR_UNSUPPORTED, "unit-pulse phantoms are not batched");
    if (p->elems.empty()) return fail(CTGPU_ERR_INVALID, "phantom has no elements");
    scanner_views(s, 0, s->nView, 0);
    if (h_angles && h_angles[k])
      for (int v = 0; v < s->nView; v++) h_angles[k][v] = s->views[v].angle;
    CUDA_TRY(upload_ray_views(s, st));
    oE[k] = total;
    total = up16(total + sizeof(PElem) * p->elems.size());
  }
  const size_t oP = total;
  total = up16(total + sizeof(RaysumLaunch) * n);
  const size_t oR = total;
  total = up16(total + sizeof(int) * (n + 1));
  ctgpu_scanner* s0 = scanners[0];
  // device buffers first: the descriptors point into them
  CUDA_TRY(ensure_device(s0->d_stage, s0->d_stage_cap, total));
  unsigned char* h = nullptr;
  int slot = 0;
  CUDA_TRY(stage_host(s0, total, &h, &slot));
  std::vector<RaysumLaunch> L(n);
  std::vector<int> rayStart(n + 1, 0);
  size_t smem = 0;
  for (int k = 0; k < n; k++) {
    ctgpu_scanner* s = scanners[k];
    const ctgpu_phantom* p = phantoms[k];
    const int nv = s->nView;
    std::memcpy(h + oE[k], p->elems.data(), sizeof(PElem) * p->elems.size());
    RaysumLaunch& q = L[k];
    q = RaysumLaunch{};
    q.geometry = s->geometry;
    q.nDet = s->nDet;
    q.nSample = s->nSample;
    q.nElem = (int)p->elems.size();
    q.nViews = nv;
    q.pitch = pitches[k];
    q.rowOffset = 0;
    q.centerDetectorLength = s->centerDetectorLength;
    q.angularDetLen = s->angularDetLen;
    q.angularDetInc = s->angularDetInc;
    q.elems = reinterpret_cast<const PElem*>(s0->d_stage + oE[k]);
    q.views = s->d_views;
    q.sdirs = s->geometry == kParallel ? s->d_sdirs : nullptr;
    q.arc = s->d_arc;
    q.arcHalf = s->d_half;
    q.sino = d_sinos[k];
    q.status = status_pointer();
    q.nSlices = 1;
    const size_t sm = raysum_prepare(q);
    if (sm > smem) smem = sm;
    rayStart[k + 1] = rayStart[k] + (nv + q.viewsPerBlock - 1) / q.viewsPerBlock;
  }
  std::memcpy(h + oP, L.data(), sizeof(RaysumLaunch) * n);
  std::memcpy(h + oR, rayStart.data(), sizeof(int) * (n + 1));
  CUDA_TRY(stage_send(s0, slot, total, st));
  cudaError_t e = launch_raysum_multi(reinterpret_cast<const RaysumLaunch*>(s0->d_stage + oP),
                                      reinterpret_cast<const int*>(s0->d_stage + oR), rayStart[n],
                                      n, smem, st);
  if (e == cudaErrorInvalidValue)
    return fail(CTGPU_ERR_UNSUPPORTED, "too many phantom elements x rays per detector for one CTA");
  CUDA_TRY(e);
  return ok();
}

int ctgpu_collect_projections_ellipsoids(ctgpu_scanner* s, const double* ell, int n, double z0,
                                         double dz, float* d_sino, int pitch, double* h_angles,
                                         void* stream) {
  if (!s || !d_sino || (n > 0 && !ell) || n < 0) return fail(CTGPU_ERR_INVALID, "null argument");
  if (pitch < s->nDet) return fail(CTGPU_ERR_INVALID, "sinogram pitch smaller than nDet");
  for (int j = 0; j < n; j++)
    if (!(ell[8 * j + 3] > 0 && ell[8 * j + 4] > 0 && ell[8 * j + 5] > 0))
      return fail(CTGPU_ERR_INVALID, "ellipsoid " + std::to_string(j) + ": semi-axes must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  scanner_views(s, 0, s->nView, 0);
  if (h_angles)
    for (int v = 0; v < s->nView; v++) h_angles[v] = s->views[v].angle;
  // ellipsoid j as the 2-D ellipse of its largest cross-section, in the
  // reference's list order (last added first), with its z extent
  std::vector<PElem> base(n > 0 ? n : 1);
  std::vector<double2> zc(n > 0 ? n : 1);
  for (int j = 0; j < n; j++) {
    const double* e = ell + 8 * j;
    base[n - 1 - j] = make_elem(kEllipse, e[0], e[1], e[3], e[4], e[6], e[7]);
    zc[n - 1 - j] = make_double2(e[2], e[5]);
  }
  CUDA_TRY(ensure_device(s->d_belems, s->d_belems_cap, base.size()));
  CUDA_TRY(ensure_device(s->d_zc, s->d_zc_cap, zc.size()));
  CUDA_TRY(ensure_device(s->d_velems, s->d_velems_cap, (size_t)(n > 0 ? n : 1) * s->nView));
  CUDA_TRY(cudaMemcpyAsync(s->d_belems, base.data(), sizeof(PElem) * base.size(),
                           cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(s->d_zc, zc.data(), sizeof(double2) * zc.size(),
                           cudaMemcpyHostToDevice, st));
  CUDA_TRY(launch_ellipsoid_sections(s->d_belems, s->d_zc, n, s->nView, z0, dz, s->d_velems, st));
  // the ray records (built and uploaded on the scanner's first call for
  // these views) after the cross-section launch, which runs meanwhile
  CUDA_TRY(upload_ray_views(s, st));
  RaysumLaunch L{};
  L.geometry = s->geometry;
  L.nDet = s->nDet;
  L.nSample = s->nSample;
  L.nElem = n;
  L.nViews = s->nView;
  L.pitch = pitch;
  L.rowOffset = 0;
  L.centerDetectorLength = s->centerDetectorLength;
  L.angularDetLen = s->angularDetLen;
  L.angularDetInc = s->angularDetInc;
  L.elems = s->d_velems;
  L.views = s->d_views;
  L.sdirs = s->d_sdirs;
  L.arc = s->d_arc;
  L.arcHalf = s->d_half;
  L.sino = d_sino;
  L.status = status_pointer();
  L.elemsPerView = 1;
  cudaError_t e = launch_raysum(L, st);
  if (e == cudaErrorInvalidValue)
    return fail(CTGPU_ERR_UNSUPPORTED, "too many ellipsoids x rays per detector for one CTA");
  CUDA_TRY(e);
  return ok();
}

int ctgpu_raysum_ellipse_gradient(ctgpu_scanner* s, const ctgpu_phantom* p,
                                  const float* d_gsino, int pitch, double* h_grad, void* stream) {
  if (!s || !p || !d_gsino || !h_grad) return fail(CTGPU_ERR_INVALID, "null argument");
  if (pitch < s->nDet) return fail(CTGPU_ERR_INVALID, "sinogram pitch smaller than nDet");
  const int n = (int)p->elems.size();
  for (const PElem& e : p->elems)
    if (e.type != kEllipse)
      return fail(CTGPU_ERR_UNSUPPORTED, "parameter gradients are defined for ellipse elements");
  if (p->unitPulse) return fail(CTGPU_ERR_UNSUPPORTED, "unit-pulse phantom");
  cudaStream_t st = (cudaStream_t)stream;
  scanner_views(s, 0, s->nView, s->offsetView);
  CUDA_TRY(const_cast<ctgpu_phantom*>(p)->upload(st));
  CUDA_TRY(upload_ray_views(s, st));
  double* d_grad = nullptr;
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d_grad), sizeof(double) * 6 * (n > 0 ? n : 1), st));
  RaysumLaunch L{};
  L.geometry = s->geometry;
  L.nDet = s->nDet;
  L.nSample = s->nSample;
  L.nElem = n;
  L.nViews = s->nView;
  L.pitch = pitch;
  L.centerDetectorLength = s->centerDetectorLength;
  L.elems = p->d_elems;
  L.views = s->d_views;
  L.sdirs = s->d_sdirs;
  L.arc = s->d_arc;
  L.arcHalf = s->d_half;
  std::vector<double> g(6 * (size_t)(n > 0 ? n : 1), 0.0);
  cudaError_t e = cudaMemsetAsync(d_grad, 0, sizeof(double) * g.size(), st);
  if (e == cudaSuccess) e = launch_raysum_ellipse_grad(L, d_gsino, d_grad, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g.data(), d_grad, sizeof(double) * g.size(), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(d_grad, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaErrorInvalidValue) return fail(CTGPU_ERR_UNSUPPORTED, "too many detectors x rays for one CTA");
  CUDA_TRY(e);
  // list index k holds the element added (n-1-k)th; rotation per degree
  for (int k = 0; k < n; k++) {
    double* o = h_grad + 6 * (size_t)(n - 1 - k);
    for (int j = 0; j < 6; j++) o[j] = g[6 * (size_t)k + j];
    o[4] *= kPi / 180.0;
  }
  return ok();
}

int ctgpu_phantom_rasterize(const ctgpu_phantom* p, int nx, int ny, double viewRatio, int nsample,
                            float* d_image, double extent[4], double increment[2], void* stream) {
  if (!p || !d_image) return fail(CTGPU_ERR_INVALID, "null argument");
  if (nx < 2 || ny < 2) return ok();   // phantom.cpp:466-467: nothing is written
  if (nsample < 1) nsample = 1;
  // phantom.cpp:473-494 (getDiameterBoundaryCircle: phantom.h:190-194)
  const double dx = p->xmax - p->xmin, dy = p->ymax - p->ymin;
  const double xcent = p->xmin + dx / 2, ycent = p->ymin + dy / 2;
  const double diam = kSqrt2 * (dx > dy ? dx : dy);
  const double half = viewRatio * (diam / kSqrt2 / 2);
  const double xmin = xcent - half, xmax = xcent + half, ymin = ycent - half, ymax = ycent + half;
  const double xinc = (xmax - xmin) / nx, yinc = (ymax - ymin) / ny;
  if (extent) { extent[0] = xmin; extent[1] = xmax; extent[2] = ymin; extent[3] = ymax; }
  if (increment) { increment[0] = xinc; increment[1] = yinc; }
  // PhantomElement ctor's phantom-to-object map (phantom.cpp:629-655)
  std::vector<RasterElem> el(p->elems.size());
  for (size_t k = 0; k < el.size(); k++) {
    const PElem& e = p->elems[k];
    M3 m = mul(mul(xlat(-e.cx, -e.cy), rotm(-e.rot)), scalem(1 / e.u, 1 / e.v));
    RasterElem r{};
    std::memcpy(r.m, m.m, sizeof(r.m));
    r.u = e.u;
    r.v = e.v;
    r.atten = e.atten;
    r.type = e.type;
    el[k] = r;
  }
  std::vector<double> xc(nx), yr(ny);
  double x = xmin;
  for (int ix = 0; ix < nx; ix++, x += xinc) xc[ix] = x;
  double y = ymin;
  for (int iy = 0; iy < ny; iy++, y += yinc) yr[iy] = y;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t be = sizeof(RasterElem) * (el.size() ? el.size() : 1);
  unsigned char* blk = nullptr;
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&blk), be + sizeof(double) * (nx + ny), st));
  cudaError_t err = cudaSuccess;
  if (!el.empty()) err = cudaMemcpyAsync(blk, el.data(), sizeof(RasterElem) * el.size(), cudaMemcpyHostToDevice, st);
  if (err == cudaSuccess) err = cudaMemcpyAsync(blk + be, xc.data(), sizeof(double) * nx, cudaMemcpyHostToDevice, st);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(blk + be + sizeof(double) * nx, yr.data(), sizeof(double) * ny, cudaMemcpyHostToDevice, st);
  RasterLaunch L{};
  L.nx = nx;
  L.ny = ny;
  L.nsample = nsample;
  L.nElem = (int)el.size();
  L.elems = reinterpret_cast<const RasterElem*>(blk);
  L.xcol = reinterpret_cast<const double*>(blk + be);
  L.yrow = reinterpret_cast<const double*>(blk + be) + nx;
  L.kxinc = xinc / nsample;
  L.kyinc = yinc / nsample;
  L.kxofs = L.kxinc / 2;
  L.kyofs = L.kyinc / 2;
  L.factor = 1.0 / static_cast<double>(nsample * nsample);
  L.image = d_image;
  if (err == cudaSuccess) err = launch_raster(L, st);
  cudaFreeAsync(blk, st);
  CUDA_TRY(err);
  return ok();
}

int ctgpu_collect_projections_host(ctgpu_scanner* s, const ctgpu_phantom* p, int startView,
                                   int nViews, int offsetView, int storageOffset, float* h_sino,
                                   double* h_angles) {
  if (!s || !p || !h_sino) return fail(CTGPU_ERR_INVALID, "null argument");
  if (storageOffset + nViews > s->nView) return fail(CTGPU_ERR_INVALID, "view range past nView");
  // rows written densely (pitch nDet), so that they come down in one copy
  const int pitch = s->nDet;
  CUDA_TRY(ensure_device(s->d_sino, s->d_sino_cap, (size_t)nViews * pitch));
  int rc = ctgpu_collect_projections(s, p, startView, nViews, offsetView, 0, s->d_sino, pitch,
                                     h_angles ? h_angles + storageOffset : nullptr, nullptr);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpy(h_sino + (size_t)storageOffset * s->nDet, s->d_sino,
                      sizeof(float) * (size_t)nViews * s->nDet, cudaMemcpyDeviceToHost));
  return ctgpu_sync(nullptr);
}

// ---------------------------------------------------------- reconstruction --
int ctgpu_recon_create(const ctgpu_geometry* g, int nx, int ny, const char* filterName,
                       double filterParam, const char* filterMethod, int zeropad,
                       const char* filterGeneration, const char* interpName, int interpFactor,
                       const char* backprojName, const ctgpu_roi* roi, ctgpu_recon** out) {
  if (!g || !out || !filterName || !filterMethod || !filterGeneration || !interpName ||
      !backprojName)
    return fail(CTGPU_ERR_INVALID, "null argument");
  if (g->geometry < 0 || g->geometry > 2)
    return fail(CTGPU_ERR_INVALID, "Unable to select a backprojection method [Backprojector::initBackprojector]");
  if (nx < 1 || ny < 1 || g->n_det < 2 || g->n_view < 1)
    return fail(CTGPU_ERR_INVALID, "image and scan sizes must be positive (nDet >= 2)");
  int fid = filter_id_from_name(filterName);
  int mid = filter_method_from_name(filterMethod);
  int gid = filter_generation_from_name(filterGeneration);
  // ProcessSignal ctor error order (procsignal.cpp:88-115)
  if (mid < 0) return fail(CTGPU_ERR_INVALID, std::string("Error creating ProcessSignal: Invalid filter method name ") + filterMethod);
  if (gid < 0) return fail(CTGPU_ERR_INVALID, std::string("Error creating ProcessSignal: Invalid frequency filter name ") + filterGeneration);
  if (fid < 0) return fail(CTGPU_ERR_INVALID, std::string("Error creating ProcessSignal: Invalid Filter name ") + filterName);
  int bp = backproj_from_name(backprojName);
  int ip = interp_from_name(interpName);
  if (bp < 0) return fail(CTGPU_ERR_INVALID, std::string("Error creating backprojector: Invalid backprojection name ") + backprojName);
  if (ip < 0) return fail(CTGPU_ERR_INVALID, std::string("Error creating backprojector: Invalid interpolation name ") + interpName);
  if (interpFactor < 1) return fail(CTGPU_ERR_INVALID, "interpolation factor must be >= 1");
  // The reference's preinterpolation factor has defined semantics only inside
  // its FFTW filter (procsignal.cpp:600-626, unavailable to pin) and scales
  // idiff's nearest index (backprojectors.cpp:627); no other path reads it.
  if (interpFactor != 1)
    return fail(CTGPU_ERR_UNSUPPORTED, "preinterpolation factor other than 1 is not supported");
  FilterSpec sp{};
  sp.filterId = fid; sp.method = mid; sp.generation = gid; sp.zeropad = zeropad;
  sp.interpFactor = interpFactor; sp.geometry = g->geometry; sp.nDet = g->n_det;
  sp.param = filterParam; sp.bandwidth = 1. / g->det_inc; sp.detInc = g->det_inc;
  sp.focalLength = g->focal_length; sp.sdl = g->source_detector_length;
  ctgpu_recon* r = new ctgpu_recon();
  std::string err;
  if (!design_filter(sp, r->fd, err)) {
    delete r;
    return fail(mid == 3 ? CTGPU_ERR_UNSUPPORTED : CTGPU_ERR_INVALID, err);
  }
  r->g = *g;
  r->nx = nx; r->ny = ny; r->interp = ip;
  r->bproj = (g->geometry == kParallel) ? bp : kTable;   // fan beams: table-derived classes (:160-163)
  r->interpFactor = interpFactor;
  r->iDetCenter = (g->n_det - 1) / 2;
  r->pitch = pitch_for(g->n_det);
  // Backproject::Backproject (backprojectors.cpp:264-319)
  r->rotScale = g->geometry == kParallel ? kPi / g->n_view : (2 * kPi) / g->n_view;
  double phmLen = g->view_diameter / kSqrt2;
  r->xMin = -phmLen / 2; r->xMax = r->xMin + phmLen;
  r->yMin = -phmLen / 2; r->yMax = r->yMin + phmLen;
  if (roi) {
    if (roi->x_min > r->xMin) r->xMin = roi->x_min;
    if (roi->x_max < r->xMax) r->xMax = roi->x_max;
    if (roi->y_min > r->yMin) r->yMin = roi->y_min;
    if (roi->y_max < r->yMax) r->yMax = roi->y_max;
    if (r->xMin > r->xMax) std::swap(r->xMin, r->xMax);
    if (r->yMin > r->yMax) std::swap(r->yMin, r->yMax);
  }
  r->xInc = (r->xMax - r->xMin) / nx;
  r->yInc = (r->yMax - r->yMin) / ny;
  double x0 = r->xMin + r->xInc / 2, y0 = r->yMin + r->yInc / 2;
  r->startR = std::sqrt(x0 * x0 + y0 * y0);
  r->startPhi = std::atan2(y0, x0);
  FilterSpectrum fs;
  filter_spectrum(r->fd, g->n_det, fs);
  r->fftN = fs.fftN;
  const size_t ns = fs.spectrum.size(), nw = r->fd.weights.size();
  size_t c1 = 0, c2 = 0;
  cudaError_t e = ensure_device(r->d_spec, c1, 2 * ns);
  if (e == cudaSuccess) e = ensure_device(r->d_weights, c2, nw);
  if (e == cudaSuccess) e = cudaMemcpy(r->d_spec, fs.spectrum.data(), sizeof(float) * ns, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(r->d_spec + ns, fs.twiddle.data(), sizeof(float) * ns, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(r->d_weights, r->fd.weights.data(), sizeof(float) * nw, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete r;
    return fail(CTGPU_ERR_CUDA, std::string("recon_create: ") + cudaGetErrorString(e));
  }
  *out = r;
  return ok();
}

int ctgpu_recon_image_axes(const ctgpu_recon* r, double extent[4], double increment[2]) {
  if (!r) return fail(CTGPU_ERR_INVALID, "null plan");
  if (extent) { extent[0] = r->xMin; extent[1] = r->xMax; extent[2] = r->yMin; extent[3] = r->yMax; }
  if (increment) { increment[0] = r->xInc; increment[1] = r->yInc; }
  return ok();
}

void ctgpu_recon_destroy(ctgpu_recon* r) { delete r; }

// Filtering of nBatch sinograms of nViews rows each, one launch.
// narrowOk: a launch of few blocks may use the N / 8-thread transform (the
// single-slice entry point; batched launches keep one arithmetic)
// Where a filter launch may also write the interval rows of the table-family
// backprojection that follows it (FilterLaunch::rows).
struct RowsTarget {
  void* rows = nullptr;
  int interp = 0, pitch = 0;
  size_t sliceStride = 0;
};

static int recon_filter_batch(ctgpu_recon* r, const float* d_sino, int sinoPitch,
                              size_t sinoStride, int nViews, float* d_filtered, int filtPitch,
                              size_t filtStride, int nBatch, cudaStream_t st,
                              bool narrowOk = false, const RowsTarget* rows = nullptr,
                              bool* rowsWritten = nullptr) {
  FilterLaunch L{};
  if (rows) {
    L.rows = rows->rows;
    L.rowsInterp = rows->interp;
    L.rowsPitch = rows->pitch;
    L.rowsSliceStride = rows->sliceStride;
  }
  L.narrowOk = narrowOk ? 1 : 0;
  L.nDet = r->g.n_det;
  L.nViews = nViews;
  L.inPitch = sinoPitch;
  L.outPitch = filtPitch;
  L.fftN = r->fftN;
  L.spectrum = reinterpret_cast<const float2*>(r->d_spec);
  L.twiddle = reinterpret_cast<const float2*>(r->d_spec) + r->fftN;
  L.weights = r->d_weights;
  L.in = d_sino;
  L.out = d_filtered;
  L.nBatch = nBatch;
  L.inSliceStride = sinoStride;
  L.outSliceStride = filtStride;
  cudaError_t e = launch_filter(L, st, rowsWritten);
  if (e == cudaErrorInvalidValue)
    return fail(CTGPU_ERR_UNSUPPORTED, "nDet too large for the shared-memory FFT filter (at most 8192)");
  CUDA_TRY(e);
  return ok();
}

int ctgpu_recon_filter(ctgpu_recon* r, const float* d_sino, int sinoPitch, int nViews,
                       float* d_filtered, int filtPitch, void* stream) {
  if (!r || !d_sino || !d_filtered) return fail(CTGPU_ERR_INVALID, "null argument");
  if (sinoPitch < r->g.n_det || filtPitch < r->g.n_det) return fail(CTGPU_ERR_INVALID, "pitch < nDet");
  return recon_filter_batch(r, d_sino, sinoPitch, 0, nViews, d_filtered, filtPitch, 0, 1,
                            (cudaStream_t)stream, true);
}

// The backprojection launch descriptor of a plan (Backproject::Backproject's
// grid and geometry, backprojectors.cpp:264-319).
static BackprojLaunch make_launch(const ctgpu_recon* r, int nViews, int pitch,
                                  const double* d_angles, const float* d_filtered,
                                  float* d_image, int accumulate, float outScale, int nBatch,
                                  size_t filtStride, size_t imageStride) {
  BackprojLaunch L{};
  L.geometry = r->g.geometry;
  L.interp = r->interp;
  L.bproj = r->bproj;
  L.nDet = r->g.n_det;
  L.nx = r->nx;
  L.ny = r->ny;
  L.nViews = nViews;
  L.pitch = pitch;
  L.iDetCenter = r->iDetCenter;
  L.detInc = r->g.det_inc;
  L.xMin = r->xMin;
  L.yMin = r->yMin;
  L.xInc = r->xInc;
  L.yInc = r->yInc;
  L.focalLength = r->g.focal_length;
  L.sdl = r->g.source_detector_length;
  L.rotScale = r->rotScale;
  {
    double xm = std::fmax(std::fabs(r->xMin), std::fabs(r->xMax));
    double ym = std::fmax(std::fabs(r->yMin), std::fabs(r->yMax));
    L.minSourceDist = r->g.focal_length - std::sqrt(xm * xm + ym * ym);
  }
  L.angles = d_angles;
  L.filtered = d_filtered;
  L.image = d_image;
  L.nBatch = nBatch;
  L.filtSliceStride = filtStride;
  L.imageSliceStride = imageStride;
  L.accumulate = accumulate;
  L.outScale = outScale;
  L.status = status_pointer();
  return L;
}

// Backprojection of nViews filtered rows; outScale multiplies this launch's sum.
// a one-slice launch's view groups (table_view_groups on this device)
static cudaError_t set_view_groups(ctgpu_recon* r, BackprojLaunch& L) {
  if (!r->sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&r->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  L.viewGroups = table_view_groups(L, r->sms);
  return cudaSuccess;
}

// reuseScratch: the scratch whose (tile, view) records an earlier launch on
// stream st built for the same view angles (table family), or null;
// anglesOnDevice: r->d_angles already holds h_angles, ordered before st's work;
// extScratch: set-up scratch the caller sized (null: the plan's own);
// splitViews: a one-slice launch of few tiles may split its views into groups
// (table family; the single-slice entry points, not the batched ones, whose
// images stay bit-identical to one another)
static int recon_backproject_scaled(ctgpu_recon* r, const float* d_filtered, int pitch,
                                    const double* h_angles, int nViews, float* d_image,
                                    int accumulate, float outScale, cudaStream_t st,
                                    int nBatch = 1, size_t filtStride = 0,
                                    size_t imageStride = 0,
                                    const unsigned char* reuseScratch = nullptr,
                                    bool anglesOnDevice = false,
                                    unsigned char* extScratch = nullptr,
                                    bool splitViews = false, bool rowsReady = false) {
  if (nViews <= 0) {
    if (!accumulate)
      for (int b = 0; b < nBatch; b++)
        CUDA_TRY(cudaMemsetAsync(d_image + b * imageStride, 0, sizeof(float) * r->nx * r->ny, st));
    return ok();
  }
  if (nBatch > 1 && r->bproj == kDiff) {
    for (int b = 0; b < nBatch; b++) {
      int rc = recon_backproject_scaled(r, d_filtered + b * filtStride, pitch, h_angles, nViews,
                                        d_image + b * imageStride, accumulate, outScale, st, 1, 0,
                                        0, nullptr, anglesOnDevice, extScratch);
      if (rc) return rc;
    }
    return ok();
  }
  if (!anglesOnDevice) {
    CUDA_TRY(ensure_device(r->d_angles, r->d_angles_cap, (size_t)nViews));
    CUDA_TRY(cudaMemcpyAsync(r->d_angles, h_angles, sizeof(double) * nViews, cudaMemcpyHostToDevice, st));
  }
  const void* views = nullptr;
  if (r->bproj == kIDiff || r->bproj == kDiff) {
    // per-view steps in the reference's own FP64 / fixed-point arithmetic
    // (backprojectors.cpp:522-527 diff, :593-597 idiff)
    std::vector<long long> iv;
    std::vector<double> dv;
    const double scale = 4294967296.0;
    for (int v = 0; v < nViews; v++) {
      double th = h_angles[v];
      if (r->bproj == kIDiff) {
        iv.push_back(nearest_ll(r->xInc * std::cos(th) / r->g.det_inc * scale));
        iv.push_back(nearest_ll(r->yInc * std::sin(th) / r->g.det_inc * scale));
        iv.push_back(nearest_ll((r->startR * std::cos(th - r->startPhi) / r->g.det_inc + r->iDetCenter) * scale));
      } else {
        dv.push_back(r->xInc * std::cos(th) / r->g.det_inc);
        dv.push_back(r->yInc * std::sin(th) / r->g.det_inc);
        dv.push_back(r->iDetCenter + r->startR * std::cos(th - r->startPhi) / r->g.det_inc);
      }
    }
    size_t bytes = 24 * (size_t)nViews;
    CUDA_TRY(ensure_device(r->d_views, r->d_views_cap, bytes));
    CUDA_TRY(cudaMemcpyAsync(r->d_views, r->bproj == kIDiff ? (const void*)iv.data() : (const void*)dv.data(),
                             bytes, cudaMemcpyHostToDevice, st));
    views = r->d_views;
  }
  BackprojLaunch L = make_launch(r, nViews, pitch, r->d_angles, d_filtered, d_image, accumulate,
                                 outScale, nBatch, filtStride, imageStride);
  if (splitViews && nBatch == 1) CUDA_TRY(set_view_groups(r, L));
  size_t sb = backproject_scratch_bytes(L);
  unsigned char* scratch = extScratch;
  bool stable = true;
  if (!scratch) {
    const size_t capBefore = r->d_scratch_cap;
    if (sb) CUDA_TRY(ensure_device(r->d_scratch, r->d_scratch_cap, sb));
    scratch = r->d_scratch;
    stable = r->d_scratch_cap == capBefore;   // a reallocated scratch holds no records
  }
  L.reuseRecords = reuseScratch && reuseScratch == scratch && stable && r->bproj != kDiff &&
                   r->bproj != kIDiff;
  if (scratch == r->d_scratch && !L.reuseRecords) r->recKeyValid = false;   // rewritten below
  L.rowsReady = rowsReady ? 1 : 0;
  cudaError_t e = launch_backproject_views(L, views, scratch, st);
  if (e == cudaErrorInvalidValue)
    return fail(CTGPU_ERR_UNSUPPORTED, "image pixels behind the fan-beam source");
  CUDA_TRY(e);
  return ok();
}

static float raw_scale(const ctgpu_recon* r) {
  double s = 1.0;
  if (r->bproj == kTrig) s *= r->rotScale;   // per-update rotScale (backprojectors.cpp:386-397)
  if (r->g.geometry == kEquilinear) s *= r->g.focal_length * r->g.focal_length;   // 1/U^2 = FL^2/vy^2
  return (float)s;
}

int ctgpu_recon_backproject(ctgpu_recon* r, const float* d_filtered, int pitch,
                            const double* h_angles, int nViews, float* d_image, int accumulate,
                            void* stream) {
  if (!r || !d_filtered || !h_angles || !d_image) return fail(CTGPU_ERR_INVALID, "null argument");
  if (pitch < r->g.n_det || (pitch & 3)) return fail(CTGPU_ERR_INVALID, "filtered pitch must be >= nDet and a multiple of 4");
  if (((uintptr_t)d_filtered & 15) != 0) return fail(CTGPU_ERR_INVALID, "filtered rows must be 16-byte aligned");
  return recon_backproject_scaled(r, d_filtered, pitch, h_angles, nViews, d_image, accumulate,
                                  raw_scale(r), (cudaStream_t)stream, 1, 0, 0, nullptr, false,
                                  nullptr, true);
}

int ctgpu_recon_postprocess(ctgpu_recon* r, float* d_image, void* stream) {
  if (!r || !d_image) return fail(CTGPU_ERR_INVALID, "null argument");
  if (r->bproj == kTrig) return ok();   // trig scales per update (Backproject::PostProcessing)
  CUDA_TRY(launch_scale_image(d_image, (size_t)r->nx * r->ny, (float)r->rotScale, (cudaStream_t)stream));
  return ok();
}

int ctgpu_recon_run(ctgpu_recon* r, const float* d_sino, int sinoPitch, const double* h_angles,
                    int startView, int nViews, float* d_image, int flags, void* stream) {
  if (!r || !d_sino || !h_angles || !d_image) return fail(CTGPU_ERR_INVALID, "null argument");
  if (nViews <= 0) nViews = r->g.n_view - startView;   // reconstructView(start, -1)
  if (startView < 0 || startView + nViews > r->g.n_view) return fail(CTGPU_ERR_INVALID, "view range outside the projections");
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(ensure_device(r->d_filtered, r->d_filtered_cap, (size_t)nViews * r->pitch));
  bool acc = (flags & CTGPU_RUN_ACCUMULATE) != 0;
  bool post = (flags & CTGPU_RUN_POSTPROCESS) != 0;
  float scale = raw_scale(r);
  if (post && !acc && r->bproj != kTrig) scale = (float)(scale * r->rotScale);   // fused PostProcessing
  // table family: the (tile, view) records depend on the geometry and the
  // angles only, so they are built on a side stream while the filter runs;
  // the scratch is sized here as the backprojection below sizes it
  const unsigned char* recs = nullptr;
  RowsTarget rt;
  if (nViews > 0 && r->bproj != kDiff && r->bproj != kIDiff) {
    CUDA_TRY(ensure_device(r->d_angles, r->d_angles_cap, (size_t)nViews));
    CUDA_TRY(cudaMemcpyAsync(r->d_angles, h_angles + startView, sizeof(double) * nViews,
                             cudaMemcpyHostToDevice, st));
    BackprojLaunch L = make_launch(r, nViews, r->pitch, r->d_angles, r->d_filtered, d_image,
                                   acc ? 1 : 0, scale, 1, 0, 0);
    CUDA_TRY(set_view_groups(r, L));
    const size_t capBefore = r->d_scratch_cap;
    CUDA_TRY(ensure_device(r->d_scratch, r->d_scratch_cap, backproject_scratch_bytes(L)));
    if (r->d_scratch_cap != capBefore) r->recKeyValid = false;
    if (!r->s_side) CUDA_TRY(cudaStreamCreateWithFlags(&r->s_side, cudaStreamNonBlocking));
    for (cudaEvent_t& e : r->sideEv)
      if (!e) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // records of the same angles (bit for bit) are still in the scratch when
    // the last call built them and nothing has rewritten them since (slices
    // of one scan reconstructed in turn)
    const double* ang = h_angles + startView;
    const bool have = r->recKeyValid && r->recKey.size() == (size_t)nViews &&
                      std::memcmp(r->recKey.data(), ang, sizeof(double) * nViews) == 0;
    if (!have) {
      r->recKeyValid = false;
      CUDA_TRY(cudaEventRecord(r->sideEv[0], st));   // angles up; the last call's work queued
      CUDA_TRY(cudaStreamWaitEvent(r->s_side, r->sideEv[0], 0));
      cudaError_t e = launch_tile_setup(L, r->d_scratch, r->s_side);
      if (e == cudaErrorInvalidValue)
        return fail(CTGPU_ERR_UNSUPPORTED, "image pixels behind the fan-beam source");
      CUDA_TRY(e);
      CUDA_TRY(cudaEventRecord(r->sideEv[1], r->s_side));
      r->recKey.assign(ang, ang + nViews);
      r->recKeyValid = true;
    }
    recs = r->d_scratch;
    // the filter writes the interval rows after the records, in the same
    // scratch (the records' set-up does not touch them)
    size_t off = 0;
    if (table_rows_layout(L, &off, &rt.pitch, &rt.interp)) {
      rt.rows = r->d_scratch + off;
      rt.sliceStride = (size_t)nViews * rt.pitch;
    }
  }
  if (!d_sino) return fail(CTGPU_ERR_INVALID, "null argument");
  if (sinoPitch < r->g.n_det) return fail(CTGPU_ERR_INVALID, "pitch < nDet");
  bool rowsWritten = false;
  int rc = recon_filter_batch(r, d_sino + (size_t)startView * sinoPitch, sinoPitch, 0, nViews,
                              r->d_filtered, r->pitch, 0, 1, st, true, rt.rows ? &rt : nullptr,
                              &rowsWritten);
  if (rc) return rc;
  if (recs) CUDA_TRY(cudaStreamWaitEvent(st, r->sideEv[1], 0));
  rc = recon_backproject_scaled(r, r->d_filtered, r->pitch, h_angles + startView, nViews, d_image,
                                acc ? 1 : 0, scale, st, 1, 0, 0, recs, recs != nullptr, nullptr,
                                true, rowsWritten);
  if (rc) return rc;
  if (post && acc) return ctgpu_recon_postprocess(r, d_image, stream);
  return ok();
}

int ctgpu_recon_run_host(ctgpu_recon* r, const float* h_sino, const double* h_angles,
                         float* h_image) {
  if (!r || !h_sino || !h_angles || !h_image) return fail(CTGPU_ERR_INVALID, "null argument");
  const int nDet = r->g.n_det, nView = r->g.n_view;
  CUDA_TRY(ensure_device(r->d_sino, r->d_sino_cap, (size_t)nView * r->pitch));
  CUDA_TRY(ensure_device(r->d_image, r->d_image_cap, (size_t)r->nx * r->ny));
  // one dense copy (the filter reads rows at pitch nDet); measured, one
  // 733 x 720 -> 512^2 slice per call: a pageable 2-D copy into the padded
  // layout 0.285 ms per call, the dense copy 0.26 ms
  CUDA_TRY(cudaMemcpy(r->d_sino, h_sino, sizeof(float) * (size_t)nDet * nView,
                      cudaMemcpyHostToDevice));
  int rc = ctgpu_recon_run(r, r->d_sino, nDet, h_angles, 0, nView, r->d_image,
                           CTGPU_RUN_POSTPROCESS, nullptr);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpy(h_image, r->d_image, sizeof(float) * r->nx * r->ny, cudaMemcpyDeviceToHost));
  return ctgpu_sync(nullptr);
}

// filtered rows and set-up scratch of one host-batch chunk, sized by the caller
struct ChunkBufs {
  float* filtered;
  unsigned char* scratch;
};
static int recon_run_batch(ctgpu_recon* r, int nBatch, const float* d_sinos, int sinoPitch,
                           long long sinoSliceStride, const double* h_angles, float* d_images,
                           long long imageSliceStride, int flags, cudaStream_t st,
                           const unsigned char* reuseScratch, bool anglesOnDevice,
                           const ChunkBufs* bufs = nullptr);

int ctgpu_recon_run_batch(ctgpu_recon* r, int nBatch, const float* d_sinos, int sinoPitch,
                          long long sinoSliceStride, const double* h_angles, float* d_images,
                          long long imageSliceStride, int flags, void* stream) {
  return recon_run_batch(r, nBatch, d_sinos, sinoPitch, sinoSliceStride, h_angles, d_images,
                         imageSliceStride, flags, (cudaStream_t)stream, nullptr, false);
}

static int recon_run_batch(ctgpu_recon* r, int nBatch, const float* d_sinos, int sinoPitch,
                           long long sinoSliceStride, const double* h_angles, float* d_images,
                           long long imageSliceStride, int flags, cudaStream_t st,
                           const unsigned char* reuseScratch, bool anglesOnDevice,
                           const ChunkBufs* bufs) {
  if (!r || !d_sinos || !h_angles || !d_images) return fail(CTGPU_ERR_INVALID, "null argument");
  if (nBatch < 1) return fail(CTGPU_ERR_INVALID, "batch size must be >= 1");
  const int nView = r->g.n_view;
  if (sinoPitch < r->g.n_det || sinoSliceStride < (long long)sinoPitch * nView ||
      imageSliceStride < (long long)r->nx * r->ny)
    return fail(CTGPU_ERR_INVALID, "pitch / slice strides too small");
  if (flags & CTGPU_RUN_ACCUMULATE) return fail(CTGPU_ERR_UNSUPPORTED, "batched runs overwrite their images");
  size_t fStride = (size_t)nView * r->pitch;
  float* filtered = bufs ? bufs->filtered : nullptr;
  if (!filtered) {
    CUDA_TRY(ensure_device(r->d_filtered, r->d_filtered_cap, fStride * nBatch));
    filtered = r->d_filtered;
  }
  // The table family's scratch (records, then interval rows) comes first, so
  // that the filter launch can write the rows from its own output and the
  // backprojection skips its row pass.
  unsigned char* scratch = bufs ? bufs->scratch : nullptr;
  RowsTarget rt;
  if (r->bproj != kDiff && r->bproj != kIDiff) {
    BackprojLaunch L = make_launch(r, nView, r->pitch, nullptr, filtered, d_images, 0, 1.f,
                                   nBatch, fStride, (size_t)imageSliceStride);
    size_t off = 0;
    if (table_rows_layout(L, &off, &rt.pitch, &rt.interp)) {
      if (!scratch) {
        const size_t sb = backproject_scratch_bytes(L);
        const size_t capBefore = r->d_scratch_cap;
        CUDA_TRY(ensure_device(r->d_scratch, r->d_scratch_cap, sb));
        r->recKeyValid = false;   // its records are rebuilt for this batch
        // a reallocated scratch holds no records for reuseScratch
        if (r->d_scratch_cap != capBefore) reuseScratch = nullptr;
        scratch = r->d_scratch;
      }
      rt.rows = scratch + off;
      rt.sliceStride = (size_t)nView * rt.pitch;
    }
  }
  bool rowsWritten = false;
  int rc = recon_filter_batch(r, d_sinos, sinoPitch, (size_t)sinoSliceStride, nView,
                              filtered, r->pitch, fStride, nBatch, st, false,
                              rt.rows ? &rt : nullptr, &rowsWritten);
  if (rc) return rc;
  float scale = raw_scale(r);
  bool post = (flags & CTGPU_RUN_POSTPROCESS) != 0;
  if (post && r->bproj != kTrig) scale = (float)(scale * r->rotScale);
  return recon_backproject_scaled(r, filtered, r->pitch, h_angles, nView, d_images, 0, scale,
                                  st, nBatch, fStride, (size_t)imageSliceStride, reuseScratch,
                                  anglesOnDevice, scratch, false, rowsWritten);
}

// Chunk sizes of a host-buffer batch.  Consecutive chunks run on two compute
// streams, so the device stays busy across chunk boundaries: a chunk costs its
// blocks' share of the resident slots (s * tiles / resident waves) plus a
// small fixed cost.  Exposed are the first chunk's input copy, the last
// chunk's output copy, a wait wherever a chunk's input copy outlasts the
// previous chunk's compute, and the second-to-last chunk's output copy where it
// outlasts the last chunk's compute.  A dynamic program over (slices covered,
// last chunk size) minimises the sum, in milliseconds from GB300 rates
// (1.35e12 pixel-view updates/s, 200 GB/s host to device, 180 GB/s back,
// 30 us per chunk).  Chunks hold at least minChunk slices (a full wave of
// tiles: smaller ones leave the SMs they cannot fill idle, e.g. 1 + 31 + 31
// + 1 slices of 512^2 took 9.54 ms against 9.37 ms for 2 + 30 + 30 + 2) and
// at most maxChunk (larger ones measured slower: 1 + 17 + 44 + 2 9.46 ms,
// 64 10.06 ms, 4 + 28 + 28 + 4 9.34 ms).  For 64 slices of 512^2 it picks
// 3 + 30 + 28 + 3.
static std::vector<int> plan_chunks(int nBatch, int maxChunk, int minChunk,
                                    long long tilesPerSlice, long long resident, double waveMs,
                                    double inMs, double outMs) {
  const int S = std::max(1, std::min(maxChunk, nBatch));
  minChunk = std::max(1, std::min(minChunk, S));   // the staging cap comes first
  if (nBatch <= minChunk) return std::vector<int>(1, nBatch);
  auto comp = [&](int sz) { return (double)(tilesPerSlice * sz) / resident * waveMs + 0.03; };
  const double inf = 1e300;
  // f[i * (S + 1) + s]: the first i slices covered, the last chunk of size s
  std::vector<double> f((size_t)(nBatch + 1) * (S + 1), inf);
  std::vector<int> prev((size_t)(nBatch + 1) * (S + 1), 0);
  auto at = [&](int i, int sz) { return (size_t)i * (S + 1) + sz; };
  for (int sz = minChunk; sz <= S; sz++) f[at(sz, sz)] = inMs * sz + comp(sz);
  for (int i = 1; i < nBatch; i++)
    for (int sz = 1; sz <= std::min(S, i); sz++) {
      const double base = f[at(i, sz)];
      if (base >= inf) continue;
      for (int s2 = minChunk; s2 <= std::min(S, nBatch - i); s2++) {
        const double c = base + comp(s2) + std::max(0.0, inMs * s2 - comp(sz));
        if (c < f[at(i + s2, s2)]) {
          f[at(i + s2, s2)] = c;
          prev[at(i + s2, s2)] = sz;
        }
      }
    }
  double best = inf;
  int last = 0;
  for (int sz = 1; sz <= S; sz++) {
    if (f[at(nBatch, sz)] >= inf) continue;
    const int p = prev[at(nBatch, sz)];
    const double c = f[at(nBatch, sz)] + outMs * sz + (p ? std::max(0.0, outMs * p - comp(sz)) : 0.0);
    if (c < best) {
      best = c;
      last = sz;
    }
  }
  if (last == 0) return std::vector<int>(1, nBatch);   // no split obeys the bounds
  std::vector<int> sizes;
  for (int i = nBatch, sz = last; i > 0;) {
    sizes.push_back(sz);
    const int p = prev[at(i, sz)];
    i -= sz;
    sz = p;
  }
  std::reverse(sizes.begin(), sizes.end());
  return sizes;
}

// the chunks of a host-buffer batch of nBatch slices on the current device
// (the plan's last answer when asked again)
static cudaError_t host_chunk_sizes(const ctgpu_recon* r, int nBatch, std::vector<int>* sizes) {
  int dev = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 != cudaSuccess) return e0;
  if (r->plannedFor == nBatch && r->plannedDev == dev) {
    *sizes = r->plannedChunks;
    return cudaSuccess;
  }
  const int nView = r->g.n_view;
  const size_t sStride = (size_t)nView * r->g.n_det, iStride = (size_t)r->nx * r->ny;
  int sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  // at most 64 slices and 1 GiB of staging per chunk buffer
  const size_t sliceBytes = sizeof(float) * (sStride + iStride);
  const int maxChunk = (int)std::max<size_t>(1, std::min<size_t>(64, (1ull << 30) / sliceBytes));
  const long long tilesPerSlice = (long long)((r->nx + kBackprojTile - 1) / kBackprojTile) *
                                  ((r->ny + kBackprojTile - 1) / kBackprojTile);
  const long long resident = (long long)sms * backproject_table_ctas_per_sm();
  const double waveMs = (double)resident * kBackprojTile * kBackprojTile * nView / 1.35e9;
  // a chunk fills the resident blocks at least once and spans at most about
  // 13 waves of them
  const int minChunk = (int)std::max<long long>(1, (resident + tilesPerSlice - 1) / tilesPerSlice);
  const int waveCap = (int)std::min<long long>(64, std::max<long long>(minChunk,
                                                     13 * resident / tilesPerSlice));
  *sizes = plan_chunks(nBatch, std::min(maxChunk, waveCap), minChunk, tilesPerSlice, resident,
                       waveMs, sizeof(float) * sStride / 2e8, sizeof(float) * iStride / 1.8e8);
  r->plannedChunks = *sizes;
  r->plannedFor = nBatch;
  r->plannedDev = dev;
  return cudaSuccess;
}

// the caller's chunk sizes, repeated from the start until n_batch slices are
// covered (the last one cut short), or the planned ones
static cudaError_t host_chunks_for(const ctgpu_recon* r, int nBatch, std::vector<int>* sizes) {
  if (r->hostChunks.empty()) return host_chunk_sizes(r, nBatch, sizes);
  sizes->clear();
  for (int left = nBatch, k = 0; left > 0; k++) {
    const int n = std::min(left, r->hostChunks[k % r->hostChunks.size()]);
    sizes->push_back(n);
    left -= n;
  }
  return cudaSuccess;
}

int ctgpu_recon_set_host_chunks(ctgpu_recon* r, const int* sizes, int n) {
  if (!r || (n > 0 && !sizes) || n < 0) return fail(CTGPU_ERR_INVALID, "null argument");
  for (int i = 0; i < n; i++)
    if (sizes[i] < 1) return fail(CTGPU_ERR_INVALID, "chunk sizes must be >= 1");
  r->hostChunks.assign(sizes, sizes + n);
  return ok();
}

int ctgpu_recon_host_chunks(const ctgpu_recon* r, int nBatch, int* sizes, int maxSizes) {
  if (!r || (!sizes && maxSizes > 0)) return fail(CTGPU_ERR_INVALID, "null argument");
  if (nBatch < 1) return fail(CTGPU_ERR_INVALID, "batch size must be >= 1");
  std::vector<int> v;
  CUDA_TRY(host_chunks_for(r, nBatch, &v));
  for (int i = 0; i < (int)v.size() && i < maxSizes; i++) sizes[i] = v[i];
  return (int)v.size();
}

int ctgpu_recon_run_batch_host(ctgpu_recon* r, int nBatch, const float* h_sinos,
                               const double* h_angles, float* h_images, int flags) {
  if (!r || !h_sinos || !h_angles || !h_images) return fail(CTGPU_ERR_INVALID, "null argument");
  if (nBatch < 1) return fail(CTGPU_ERR_INVALID, "batch size must be >= 1");
  if (flags & CTGPU_RUN_ACCUMULATE) return fail(CTGPU_ERR_UNSUPPORTED, "batched runs overwrite their images");
  const int nDet = r->g.n_det, nView = r->g.n_view;
  // input rows arrive dense ([slice][view][n_det], one plain copy per chunk);
  // the filter reads them at pitch n_det and writes the aligned filtered rows
  const size_t sStride = (size_t)nView * nDet, iStride = (size_t)r->nx * r->ny;
  std::vector<int> sizes;
  CUDA_TRY(host_chunks_for(r, nBatch, &sizes));
  std::vector<int> first;
  int chunk = 0;
  for (size_t c = 0, at = 0; c < sizes.size(); at += sizes[c], c++) {
    first.push_back((int)at);
    chunk = std::max(chunk, sizes[c]);
  }
  CUDA_TRY(ensure_device(r->d_bsino, r->d_bsino_cap, 2 * chunk * sStride));
  CUDA_TRY(ensure_device(r->d_bimage, r->d_bimage_cap, 2 * chunk * iStride));
  if (r->h_angles_cap < (size_t)nView) {
    if (r->h_angles_pinned) cudaFreeHost(r->h_angles_pinned);
    r->h_angles_pinned = nullptr;
    r->h_angles_cap = 0;
    CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&r->h_angles_pinned),
                           sizeof(double) * (nView ? nView : 1), cudaHostAllocDefault));
    r->h_angles_cap = nView;
  }
  for (cudaStream_t* s : {&r->s_in, &r->s_comp, &r->s_out, &r->s_comp2})
    if (!*s) CUDA_TRY(cudaStreamCreateWithFlags(s, cudaStreamNonBlocking));
  for (cudaEvent_t& e : r->ev)
    if (!e) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  // the angles go up once, from page-locked memory, on the input stream ahead
  // of the first chunk (the last call's copies are done: each call ends
  // synchronised).  Uploaded per chunk on the compute stream, a chunk's
  // angles queued behind the next chunk's input copy in the same direction.
  std::memcpy(r->h_angles_pinned, h_angles, sizeof(double) * nView);
  CUDA_TRY(ensure_device(r->d_angles, r->d_angles_cap, (size_t)nView));
  CUDA_TRY(cudaMemcpyAsync(r->d_angles, r->h_angles_pinned, sizeof(double) * nView,
                           cudaMemcpyHostToDevice, r->s_in));
  cudaEvent_t* inDone = r->ev;
  cudaEvent_t* compDone = r->ev + 2;
  cudaEvent_t* outDone = r->ev + 4;
  const int nChunks = (int)sizes.size();
  // two sets of filtered rows and set-up scratch, one per compute stream,
  // each sized for the largest chunk up front: no buffer is reallocated (a
  // synchronising free) between chunks, and each set's records stay put
  ChunkBufs bufs[2];
  cudaStream_t comp[2] = {r->s_comp, r->s_comp2};
  const unsigned char* recScratch[2] = {nullptr, nullptr};
  {
    const size_t fStride = (size_t)nView * r->pitch;
    const int sets = nChunks > 1 ? 2 : 1;
    CUDA_TRY(ensure_device(r->d_filtered, r->d_filtered_cap, fStride * chunk));
    if (sets > 1) CUDA_TRY(ensure_device(r->d_filtered2, r->d_filtered2_cap, fStride * chunk));
    BackprojLaunch L = make_launch(r, nView, r->pitch, nullptr, nullptr, nullptr, 0, 1.f, chunk,
                                   fStride, iStride);
    const size_t sb = backproject_scratch_bytes(L);
    CUDA_TRY(ensure_device(r->d_scratch, r->d_scratch_cap, sb ? sb : 1));
    r->recKeyValid = false;   // the chunks rebuild its records
    if (sets > 1) CUDA_TRY(ensure_device(r->d_scratch2, r->d_scratch2_cap, sb ? sb : 1));
    bufs[0] = ChunkBufs{r->d_filtered, r->d_scratch};
    bufs[1] = ChunkBufs{r->d_filtered2, r->d_scratch2};
  }
  // image copy of chunk c, issued one iteration late so that a pageable
  // destination (whose copy blocks the host) does not hold back the next
  // chunk's input copy and launch
  auto copy_out = [&](int c) -> int {
    const int b = c & 1;
    CUDA_TRY(cudaStreamWaitEvent(r->s_out, compDone[b], 0));
    CUDA_TRY(cudaMemcpyAsync(h_images + (size_t)first[c] * iStride, r->d_bimage + b * chunk * iStride,
                             sizeof(float) * iStride * sizes[c], cudaMemcpyDeviceToHost, r->s_out));
    CUDA_TRY(cudaEventRecord(outDone[b], r->s_out));
    return CTGPU_OK;
  };
  // chunk c runs on compute stream c & 1 with buffer set c & 1: the next
  // chunk's filter and backprojection start in this one's tail
  for (int c = 0; c < nChunks; c++) {
    const int b = c & 1, n = sizes[c];
    float* dS = r->d_bsino + b * chunk * sStride;
    float* dI = r->d_bimage + b * chunk * iStride;
    if (c >= 2) CUDA_TRY(cudaStreamWaitEvent(r->s_in, compDone[b], 0));   // buffer b read
    CUDA_TRY(cudaMemcpyAsync(dS, h_sinos + (size_t)first[c] * sStride, sizeof(float) * sStride * n,
                             cudaMemcpyHostToDevice, r->s_in));
    CUDA_TRY(cudaEventRecord(inDone[b], r->s_in));
    CUDA_TRY(cudaStreamWaitEvent(comp[b], inDone[b], 0));
    if (c >= 2) CUDA_TRY(cudaStreamWaitEvent(comp[b], outDone[b], 0));   // image b copied out
    // every chunk has the same view angles: the first chunk of each set
    // builds its (tile, view) records, the set's later chunks (same stream)
    // use them
    int rc = recon_run_batch(r, n, dS, nDet, (long long)sStride, r->h_angles_pinned, dI,
                             (long long)iStride, flags & CTGPU_RUN_POSTPROCESS, comp[b],
                             recScratch[b], true, &bufs[b]);
    if (rc) return rc;
    recScratch[b] = bufs[b].scratch;
    CUDA_TRY(cudaEventRecord(compDone[b], comp[b]));
    if (c >= 1 && (rc = copy_out(c - 1))) return rc;
  }
  int rc = copy_out(nChunks - 1);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(r->s_out));   // after every chunk's compute
  CUDA_TRY(cudaStreamSynchronize(r->s_comp2));
  return ctgpu_sync(r->s_comp);
}

int ctgpu_recon_backproject_batch(ctgpu_recon* r, int nBatch, const float* d_filtered, int pitch,
                                  long long filtSliceStride, const double* h_angles, int nViews,
                                  float* d_images, long long imageSliceStride, int flags,
                                  void* stream) {
  if (!r || !d_filtered || !h_angles || !d_images) return fail(CTGPU_ERR_INVALID, "null argument");
  if (nBatch < 1) return fail(CTGPU_ERR_INVALID, "batch size must be >= 1");
  if (pitch < r->g.n_det || (pitch & 3) || (filtSliceStride & 3) ||
      ((uintptr_t)d_filtered & 15) != 0)
    return fail(CTGPU_ERR_INVALID, "filtered rows must be 16-byte aligned (pitch and slice stride multiples of 4)");
  if (filtSliceStride < (long long)pitch * nViews || imageSliceStride < (long long)r->nx * r->ny)
    return fail(CTGPU_ERR_INVALID, "slice strides too small");
  if (flags & CTGPU_RUN_ACCUMULATE) return fail(CTGPU_ERR_UNSUPPORTED, "batched launches overwrite their images");
  float scale = raw_scale(r);
  if ((flags & CTGPU_RUN_POSTPROCESS) && r->bproj != kTrig) scale = (float)(scale * r->rotScale);
  return recon_backproject_scaled(r, d_filtered, pitch, h_angles, nViews, d_images, 0, scale,
                                  (cudaStream_t)stream, nBatch, (size_t)filtSliceStride,
                                  (size_t)imageSliceStride);
}

int ctgpu_recon_project(ctgpu_recon* r, const float* d_image, const double* h_angles, int nViews,
                        float* d_sino, int pitch, float scale, void* stream) {
  if (!r || !d_image || !h_angles || !d_sino) return fail(CTGPU_ERR_INVALID, "null argument");
  if (r->g.geometry != kParallel || r->interp != kLinear || r->bproj != kTable)
    return fail(CTGPU_ERR_UNSUPPORTED, "projector: parallel geometry, table backprojector, linear interpolation");
  if (pitch < r->g.n_det) return fail(CTGPU_ERR_INVALID, "pitch < nDet");
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(ensure_device(r->d_angles, r->d_angles_cap, (size_t)nViews));
  CUDA_TRY(cudaMemcpyAsync(r->d_angles, h_angles, sizeof(double) * nViews, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemset2DAsync(d_sino, sizeof(float) * pitch, 0, sizeof(float) * r->g.n_det, nViews, st));
  BackprojLaunch L{};
  L.geometry = kParallel;
  L.interp = kLinear;
  L.bproj = kTable;
  L.nDet = r->g.n_det;
  L.nx = r->nx;
  L.ny = r->ny;
  L.nViews = nViews;
  L.pitch = pitch;
  L.iDetCenter = r->iDetCenter;
  L.detInc = r->g.det_inc;
  L.xMin = r->xMin;
  L.yMin = r->yMin;
  L.xInc = r->xInc;
  L.yInc = r->yInc;
  L.angles = r->d_angles;
  L.nBatch = 1;
  L.status = status_pointer();
  CUDA_TRY(launch_project_table(L, d_image, d_sino, scale, st));
  return ok();
}

// ----------------------------------------------------------------- helical --
// eql: the equilinear restatement (true fan angles), which the reference does
// not have; otherwise the reference's checks and messages (projections.cpp:203-229)
static int helical_check(const ctgpu_geometry* g, int nViewIn, int interpView, int* last,
                         int* offset, bool eql) {
  if (!g) return fail(CTGPU_ERR_INVALID, "null geometry");
  if (eql) {
    if (g->geometry != kEquilinear)
      return fail(CTGPU_ERR_INVALID, "the equilinear 180LI needs equilinear projections");
  } else if (g->geometry != kEquiangular) {
    if (g->geometry == kParallel) return fail(CTGPU_ERR_INVALID, "Helical 180LI not yet implemented for PARALLEL geometry");
    if (g->geometry == kEquilinear) return fail(CTGPU_ERR_INVALID, "Helical 180LI not yet implemented for EQUILINEAR geometry");
    return fail(CTGPU_ERR_INVALID, "Invalid geometry in projection data file");
  }
  double dbeta = g->rot_inc, fan = g->fan_beam_angle;
  if (nViewIn < (int)((2 * (kPi + fan)) / dbeta) - 1)
    return fail(CTGPU_ERR_INVALID, "Data set does not include 360 +2*FanBeamAngle views");
  *offset = 0;
  if (interpView >= 0) {
    if (interpView * dbeta < kPi + fan || interpView * dbeta + kPi + fan > nViewIn * dbeta)
      return fail(CTGPU_ERR_INVALID, "There isn't PI+fanAngle of data on either side of the requested interpolation view");
    *offset = interpView - (int)((kPi + fan) / dbeta);
  }
  *last = (int)((kPi + fan) / dbeta);
  if (*offset + 2 * *last >= nViewIn)
    return fail(CTGPU_ERR_INVALID, "Data set does not include 360 +2*FanBeamAngle views");
  return ok();
}

static int helical_size(const ctgpu_geometry* g, int nViewIn, int interpView, int* nOut, bool eql) {
  int last, off;
  int rc = helical_check(g, nViewIn, interpView, &last, &off, eql);
  if (rc) return rc;
  if (nOut) *nOut = last + 1;
  return ok();
}

static int helical_run(const ctgpu_geometry* g, const float* d_in, int nViewIn, int interpView,
                       float* d_out, int pitch, double* h_angles, int* nOut, void* stream,
                       bool eql) {
  int last, off;
  int rc = helical_check(g, nViewIn, interpView, &last, &off, eql);
  if (rc) return rc;
  if (!d_in || !d_out || pitch < g->n_det) return fail(CTGPU_ERR_INVALID, "bad buffers");
  HelicalLaunch L{};
  L.nDet = g->n_det;
  L.nViewIn = nViewIn;
  L.nViewOut = last + 1;
  L.offsetView = off;
  L.pitch = pitch;
  L.dbeta = g->rot_inc;
  L.dgamma = g->det_inc;
  L.fan = g->fan_beam_angle;
  L.equilinear = eql ? 1 : 0;
  L.sdl = g->source_detector_length;
  L.in = d_in;
  L.out = d_out;
  L.status = status_pointer();
  CUDA_TRY(launch_helical180li(L, (cudaStream_t)stream));
  if (h_angles)
    for (int i = 0; i <= last; i++) h_angles[i] = (i + off) * g->rot_inc;
  if (nOut) *nOut = last + 1;
  return ok();
}

static int feather_run(const ctgpu_geometry* g, float* d_data, int nView, int pitch, void* stream,
                       bool eql) {
  if (!g || !d_data) return fail(CTGPU_ERR_INVALID, "null argument");
  double dbeta = g->rot_inc, fan = g->fan_beam_angle;
  if (nView != (int)((kPi + fan) / dbeta) + 1)   // projections.cpp:377-389
    return fail(CTGPU_ERR_INVALID, "Data set does seem have enough data to be a halfscan data set");
  if (g->geometry == kParallel) return fail(CTGPU_ERR_INVALID, "HalfScanFeather not yet implemented for PARALLEL geometry");
  if (g->geometry != kEquiangular && g->geometry != kEquilinear) return fail(CTGPU_ERR_INVALID, "Invalid geometry");
  if (eql && g->geometry != kEquilinear)
    return fail(CTGPU_ERR_INVALID, "the equilinear feathering needs equilinear projections");
  cudaStream_t st = (cudaStream_t)stream;
  float* tmp = nullptr;
  size_t bytes = sizeof(float) * (size_t)nView * pitch;
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&tmp), bytes, st));
  cudaError_t e = cudaMemcpyAsync(tmp, d_data, bytes, cudaMemcpyDeviceToDevice, st);
  HelicalLaunch L{};
  L.nDet = g->n_det;
  L.nViewIn = nView;
  L.nViewOut = nView;
  L.pitch = pitch;
  L.dbeta = dbeta;
  L.dgamma = g->det_inc;
  L.fan = fan;
  L.equilinear = eql ? 1 : 0;
  L.sdl = g->source_detector_length;
  L.in = tmp;
  L.out = d_data;
  L.status = status_pointer();
  if (e == cudaSuccess) e = launch_halfscan_feather(L, st);
  cudaFreeAsync(tmp, st);
  CUDA_TRY(e);
  return ok();
}

int ctgpu_helical180li_size(const ctgpu_geometry* g, int nViewIn, int interpView, int* nOut) {
  return helical_size(g, nViewIn, interpView, nOut, false);
}

int ctgpu_helical180li(const ctgpu_geometry* g, const float* d_in, int nViewIn, int interpView,
                       float* d_out, int pitch, double* h_angles, int* nOut, void* stream) {
  return helical_run(g, d_in, nViewIn, interpView, d_out, pitch, h_angles, nOut, stream, false);
}

int ctgpu_halfscan_feather(const ctgpu_geometry* g, float* d_data, int nView, int pitch,
                           void* stream) {
  return feather_run(g, d_data, nView, pitch, stream, false);
}

int ctgpu_helical180li_equilinear_size(const ctgpu_geometry* g, int nViewIn, int interpView,
                                       int* nOut) {
  return helical_size(g, nViewIn, interpView, nOut, true);
}

int ctgpu_helical180li_equilinear(const ctgpu_geometry* g, const float* d_in, int nViewIn,
                                  int interpView, float* d_out, int pitch, double* h_angles,
                                  int* nOut, void* stream) {
  return helical_run(g, d_in, nViewIn, interpView, d_out, pitch, h_angles, nOut, stream, true);
}

int ctgpu_halfscan_feather_equilinear(const ctgpu_geometry* g, float* d_data, int nView,
                                      int pitch, void* stream) {
  return feather_run(g, d_data, nView, pitch, stream, true);
}

}  // extern "C"

extern "C" {

// Projections::interpolateToParallel (projections.cpp:1250-1328): the host
// builds the reference's FP64 tables (fan angle and t = FL sin(gamma) of each
// detector, accumulated output angles and positions), the device sorts and
// interpolates (k_rebin.cu).
int ctgpu_interpolate_to_parallel(const ctgpu_geometry* g, const float* d_sino, int pitch,
                                  const double* h_angles, float* d_out, int outPitch,
                                  ctgpu_geometry* gOut, double* h_outAngles, void* stream) {
  if (!g || !d_sino || !h_angles || !d_out || !gOut || !h_outAngles)
    return fail(CTGPU_ERR_INVALID, "null argument");
  const int nDet = g->n_det, nView = g->n_view;
  if (nDet < 1 || nView < 1 || pitch < nDet || outPitch < nDet)
    return fail(CTGPU_ERR_INVALID, "bad sizes");
  cudaStream_t st = (cudaStream_t)stream;
  if (g->geometry == kParallel) {   // returns the projections themselves
    *gOut = *g;
    for (int v = 0; v < nView; v++) h_outAngles[v] = h_angles[v];
    CUDA_TRY(cudaMemcpy2DAsync(d_out, sizeof(float) * outPitch, d_sino, sizeof(float) * pitch,
                               sizeof(float) * nDet, nView, cudaMemcpyDeviceToDevice, st));
    return ok();
  }
  if (g->geometry != kEquiangular && g->geometry != kEquilinear)
    return fail(CTGPU_ERR_INVALID, "Invalid geometry");
  if (rebin_sort_bytes(nView) > 200 * 1024)
    return fail(CTGPU_ERR_UNSUPPORTED, "too many views to sort one detector's rays in shared memory");
  ctgpu_geometry o = *g;
  o.geometry = kParallel;
  o.rot_start = 0;
  o.rot_inc = 2 * kPi / nView;
  o.det_start = -g->view_diameter / 2;
  o.det_inc = g->view_diameter / nDet;
  if (nDet % 2 == 0) o.det_inc = g->view_diameter / (nDet - 1);
  std::vector<double> gam(nDet), t(nDet), tSorted(nDet), thOut(nView), posOut(nDet);
  std::vector<int> order(nDet), group(nDet);
  double dp = g->det_start;
  for (int d = 0; d < nDet; d++, dp += g->det_inc) {
    gam[d] = g->geometry == kEquilinear ? std::atan(dp / g->source_detector_length) : dp;
    t[d] = g->focal_length * std::sin(gam[d]);
    order[d] = d;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return t[a] < t[b]; });
  for (int r = 0; r < nDet; r++) {
    group[order[r]] = r;
    tSorted[r] = t[order[r]];
  }
  double a = g->rot_start;
  for (int v = 0; v < nView; v++, a += o.rot_inc) thOut[v] = a;
  double p = o.det_start;
  for (int d = 0; d < nDet; d++, p += o.det_inc) posOut[d] = p;
  // one device block: angles, gam, thetaOut, tSorted, posOut (doubles), group (ints), tmp
  const size_t nd = (size_t)nView * 2 + (size_t)nDet * 3;
  const size_t bytes = sizeof(double) * nd + sizeof(int) * nDet + 16 + sizeof(float) * (size_t)nView * nDet;
  unsigned char* blk = nullptr;
  CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&blk), bytes, st));
  double* dd = reinterpret_cast<double*>(blk);
  std::vector<double> host;
  host.reserve(nd);
  host.insert(host.end(), h_angles, h_angles + nView);
  host.insert(host.end(), gam.begin(), gam.end());
  host.insert(host.end(), thOut.begin(), thOut.end());
  host.insert(host.end(), tSorted.begin(), tSorted.end());
  host.insert(host.end(), posOut.begin(), posOut.end());
  int* di = reinterpret_cast<int*>(dd + nd);
  float* tmp = reinterpret_cast<float*>(blk + ((sizeof(double) * nd + sizeof(int) * nDet + 15) & ~(size_t)15));
  cudaError_t e = cudaMemcpyAsync(dd, host.data(), sizeof(double) * nd, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(di, group.data(), sizeof(int) * nDet, cudaMemcpyHostToDevice, st);
  RebinLaunch L{};
  L.nDet = nDet;
  L.nView = nView;
  L.pitch = pitch;
  L.outPitch = outPitch;
  L.in = d_sino;
  L.angles = dd;
  L.gam = dd + nView;
  L.thetaOut = dd + nView + nDet;
  L.tSorted = dd + 2 * nView + nDet;
  L.posOut = dd + 2 * nView + 2 * nDet;
  L.group = di;
  L.tmp = tmp;
  L.out = d_out;
  if (e == cudaSuccess) e = launch_rebin(L, st);
  cudaFreeAsync(blk, st);
  // the host tables are staged by the pageable copies before they return
  CUDA_TRY(e);
  *gOut = o;
  for (int v = 0; v < nView; v++) h_outAngles[v] = thOut[v];
  return ok();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Helical plan: Helical180LI (+ HalfScanFeather) at many interpolation views
// of one data set, tables once, one gather launch per run.
// ---------------------------------------------------------------------------
struct ctgpu_helical_plan {
  ctgpu_geometry g;
  int nViewIn = 0, nOut = 0, flags = 0;
  HelicalTap* d_interp = nullptr;
  FeatherTap* d_feather = nullptr;
  int* d_offsets = nullptr;
  size_t d_offsets_cap = 0;
  ~ctgpu_helical_plan() {
    for (void* p : {(void*)d_interp, (void*)d_feather, (void*)d_offsets})
      if (p) cudaFree(p);
  }
};

extern "C" {

int ctgpu_helical_plan_create(const ctgpu_geometry* g, int nViewIn, int flags,
                              ctgpu_helical_plan** out) {
  if (!g || !out) return fail(CTGPU_ERR_INVALID, "null argument");
  const bool eql = (flags & CTGPU_HELICAL_EQUILINEAR) != 0;
  int last, off;
  int rc = helical_check(g, nViewIn, -1, &last, &off, eql);
  if (rc) return rc;
  std::unique_ptr<ctgpu_helical_plan> p(new ctgpu_helical_plan);
  p->g = *g;
  p->nViewIn = nViewIn;
  p->nOut = last + 1;
  p->flags = flags;
  const int nDet = g->n_det;
  // fan angle per detector, FP64 on the host (projections.cpp:247; the
  // equilinear restatement maps the position through atan(pos / SDL))
  std::vector<double> gam(nDet);
  for (int id = 0; id < nDet; id++) {
    const double pos = (id - (nDet - 1) / 2) * g->det_inc;
    gam[id] = eql ? std::atan(pos / g->source_detector_length) : pos;
  }
  double* d_gam = nullptr;
  const size_t nTab = (size_t)p->nOut * nDet;
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&d_gam), sizeof(double) * nDet));
  cudaError_t e = cudaMemcpy(d_gam, gam.data(), sizeof(double) * nDet, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&p->d_interp), sizeof(HelicalTap) * nTab);
  if (e == cudaSuccess && (flags & CTGPU_HELICAL_FEATHER))
    e = cudaMalloc(reinterpret_cast<void**>(&p->d_feather), sizeof(FeatherTap) * nTab);
  if (e == cudaSuccess) {
    HelicalLaunch L{};
    L.nDet = nDet;
    L.nViewIn = nViewIn;
    L.nViewOut = p->nOut;
    L.dbeta = g->rot_inc;
    L.dgamma = g->det_inc;
    L.fan = g->fan_beam_angle;
    L.equilinear = eql ? 1 : 0;
    L.sdl = g->source_detector_length;
    e = launch_helical_tables(L, d_gam, p->d_interp, p->d_feather, nullptr);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaFree(d_gam);
  CUDA_TRY(e);
  *out = p.release();
  return ok();
}

int ctgpu_helical_plan_views(const ctgpu_helical_plan* p, int* nOut) {
  if (!p || !nOut) return fail(CTGPU_ERR_INVALID, "null argument");
  *nOut = p->nOut;
  return ok();
}

int ctgpu_helical_plan_run(ctgpu_helical_plan* p, const float* d_in, int inPitch,
                           const int* interpViews, int nSlices, float* d_out, int outPitch,
                           long long outSliceStride, double* h_angles, void* stream) {
  if (!p || !d_in || !interpViews || !d_out || nSlices < 1) return fail(CTGPU_ERR_INVALID, "null argument");
  if (inPitch < p->g.n_det || outPitch < p->g.n_det ||
      outSliceStride < (long long)outPitch * p->nOut)
    return fail(CTGPU_ERR_INVALID, "pitch / slice stride too small");
  const bool eql = (p->flags & CTGPU_HELICAL_EQUILINEAR) != 0;
  std::vector<int> offs(nSlices);
  for (int z = 0; z < nSlices; z++) {
    int last, off;
    int rc = helical_check(&p->g, p->nViewIn, interpViews[z], &last, &off, eql);
    if (rc) return rc;
    offs[z] = off;
    if (h_angles)
      for (int i = 0; i <= last; i++) h_angles[(size_t)z * p->nOut + i] = (i + off) * p->g.rot_inc;
  }
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(ensure_device(p->d_offsets, p->d_offsets_cap, (size_t)nSlices));
  CUDA_TRY(cudaMemcpyAsync(p->d_offsets, offs.data(), sizeof(int) * nSlices,
                           cudaMemcpyHostToDevice, st));
  HelicalSlicesLaunch L{};
  L.nDet = p->g.n_det;
  L.nViewOut = p->nOut;
  L.nSlices = nSlices;
  L.inPitch = inPitch;
  L.outPitch = outPitch;
  L.in = d_in;
  L.offsets = p->d_offsets;
  L.interp = p->d_interp;
  L.feather = p->d_feather;
  L.sf = p->nOut * p->g.rot_inc / kPi;   // projections.cpp:434-437
  L.out = d_out;
  L.outSliceStride = (size_t)outSliceStride;
  L.status = status_pointer();
  CUDA_TRY(launch_helical_slices(L, st));
  return ok();
}

void ctgpu_helical_plan_destroy(ctgpu_helical_plan* p) { delete p; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched reconstruction of problems of uneven sizes.  Each problem keeps a
// plan of its own (filter design, image grid, geometry) and its (tile, view)
// records, built once at create (the view angles are fixed there); at each
// run the problems' filter launches, which write the interval rows too, run
// as parallel branches on kSideStreams streams, then one persistent launch
// backprojects every (problem, tile) item, longest first.
// ---------------------------------------------------------------------------
namespace {

constexpr int kSideStreams = 4;

struct BatchEntry {
  ctgpu_recon* plan = nullptr;
  const float* d_sino = nullptr;
  int sinoPitch = 0;
  float* d_image = nullptr;
  size_t filtOff = 0, angOff = 0, scratchOff = 0;   // arena offsets
  BackprojLaunch L{};
  TablePrep prep{};
};

}  // namespace

struct ctgpu_batch {
  std::vector<BatchEntry> probs;
  std::vector<BatchItem> items;
  unsigned char* d_arena = nullptr;
  size_t arenaBytes = 0;
  BatchProblem* d_probs = nullptr;
  BatchItem* d_items = nullptr;
  int* d_counter = nullptr;
  int flags = 0;
  bool shaped = false;
  BatchShape shape{4, 16};
  int gridBlocks = 0;
  cudaStream_t side[kSideStreams] = {};
  cudaStream_t capture = nullptr;
  cudaEvent_t fork = nullptr, join[kSideStreams] = {};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~ctgpu_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& e : probs)
      if (e.plan) ctgpu_recon_destroy(e.plan);
    for (void* p : {(void*)d_arena, (void*)d_probs, (void*)d_items, (void*)d_counter})
      if (p) cudaFree(p);
    if (fork) cudaEventDestroy(fork);
    for (cudaEvent_t e : join)
      if (e) cudaEventDestroy(e);
    for (cudaStream_t s : side)
      if (s) cudaStreamDestroy(s);
    if (capture) cudaStreamDestroy(capture);
  }
};

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// problem table for a launch shape; false when a problem's window does not fit
static bool batch_table(const ctgpu_batch* b, const BatchShape& shape,
                        std::vector<BatchProblem>& out) {
  out.resize(b->probs.size());
  for (size_t i = 0; i < b->probs.size(); i++) {
    const BatchEntry& e = b->probs[i];
    BatchProblem& P = out[i];
    P.L = e.L;
    P.recs = b->d_arena + e.scratchOff;
    P.rows = b->d_arena + e.scratchOff + e.prep.recBytes;
    P.kind = e.prep.kind;
    P.win = e.prep.win;
    P.rpitch = e.prep.rpitch;
    P.elemBytes = e.prep.elemBytes;
    P.eps = e.prep.eps;
    P.fan = e.prep.fan;
    P.tilesX = (e.L.nx + 31) / 32;
    P.cv = batch_views_per_stage(e.prep, shape);
    if (P.cv < 1) return false;
  }
  return true;
}

// the problems' filter launches (their records were built at create) as
// branches forked from and joined to s
static int batch_enqueue_prep(ctgpu_batch* b, cudaStream_t s) {
  CUDA_TRY(cudaEventRecord(b->fork, s));
  for (int k = 0; k < kSideStreams; k++) CUDA_TRY(cudaStreamWaitEvent(b->side[k], b->fork, 0));
  for (size_t i = 0; i < b->probs.size(); i++) {
    BatchEntry& e = b->probs[i];
    cudaStream_t ss = b->side[i % kSideStreams];
    // the filter writes the problem's interval rows too, where its kernel can
    RowsTarget rt;
    rt.rows = b->d_arena + e.scratchOff + e.prep.recBytes;
    rt.interp = e.L.interp;
    rt.pitch = e.prep.rpitch;
    rt.sliceStride = (size_t)e.L.nViews * e.prep.rpitch;
    bool rowsWritten = false;
    int rc = recon_filter_batch(e.plan, e.d_sino, e.sinoPitch, 0, e.L.nViews,
                                reinterpret_cast<float*>(b->d_arena + e.filtOff), e.plan->pitch,
                                0, 1, ss, false, &rt, &rowsWritten);
    if (rc) return rc;
    BackprojLaunch Lp = e.L;
    Lp.rowsReady = rowsWritten ? 1 : 0;
    Lp.reuseRecords = 1;   // built at create
    CUDA_TRY(launch_table_prep(Lp, e.prep, b->d_arena + e.scratchOff, ss));
  }
  for (int k = 0; k < kSideStreams; k++) {
    CUDA_TRY(cudaEventRecord(b->join[k], b->side[k]));
    CUDA_TRY(cudaStreamWaitEvent(s, b->join[k], 0));
  }
  return ok();
}

static int batch_enqueue_backprojection(ctgpu_batch* b, cudaStream_t s) {
  CUDA_TRY(cudaMemsetAsync(b->d_counter, 0, sizeof(int), s));
  CUDA_TRY(launch_backproject_batch(b->d_probs, b->d_items, (int)b->items.size(), b->d_counter,
                                    b->shape, b->gridBlocks, status_pointer(), s));
  return ok();
}

static int batch_set_shape(ctgpu_batch* b, const BatchShape& shape) {
  std::vector<BatchProblem> table;
  if (!batch_table(b, shape, table)) return fail(CTGPU_ERR_UNSUPPORTED, "shape does not fit");
  CUDA_TRY(prepare_backproject_batch(shape, &b->gridBlocks));
  CUDA_TRY(cudaMemcpy(b->d_probs, table.data(), sizeof(BatchProblem) * table.size(),
                      cudaMemcpyHostToDevice));
  b->shape = shape;
  return ok();
}

// Autotuner: every candidate launch shape that fits is timed on this batch
// (prepared data, one warm-up and two timed launches, the faster kept) and
// the fastest is kept.
static int batch_tune(ctgpu_batch* b, cudaStream_t s) {
  static const BatchShape cands[] = {{4, 16}, {4, 8}, {3, 16}, {2, 16}};
  cudaEvent_t t0, t1;
  CUDA_TRY(cudaEventCreate(&t0));
  CUDA_TRY(cudaEventCreate(&t1));
  float best = 1e30f;
  BatchShape bestShape{0, 0};
  int rc = ok();
  for (const BatchShape& c : cands) {
    if (batch_set_shape(b, c) != CTGPU_OK) continue;
    float ms = 1e30f;
    for (int rep = 0; rep < 3 && rc == CTGPU_OK; rep++) {
      if (cudaEventRecord(t0, s) != cudaSuccess) rc = fail(CTGPU_ERR_CUDA, "event");
      if (rc == CTGPU_OK) rc = batch_enqueue_backprojection(b, s);
      if (rc == CTGPU_OK && cudaEventRecord(t1, s) != cudaSuccess) rc = fail(CTGPU_ERR_CUDA, "event");
      if (rc == CTGPU_OK) rc = ctgpu_sync(s);
      float t = 0.f;
      if (rc == CTGPU_OK && rep > 0 && cudaEventElapsedTime(&t, t0, t1) == cudaSuccess && t < ms)
        ms = t;
    }
    if (rc != CTGPU_OK) break;
    if (ms < best) {
      best = ms;
      bestShape = c;
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (rc != CTGPU_OK) return rc;
  if (bestShape.blocksPerSM == 0)
    return fail(CTGPU_ERR_UNSUPPORTED, "a problem's tile window is too wide for the batched path");
  return batch_set_shape(b, bestShape);
}

extern "C" {

int ctgpu_batch_create(const ctgpu_batch_problem* problems, int n, int flags, ctgpu_batch** out) {
  if (!problems || !out || n < 1) return fail(CTGPU_ERR_INVALID, "null argument or empty batch");
  std::unique_ptr<ctgpu_batch> b(new ctgpu_batch);
  b->flags = flags;
  b->probs.resize(n);
  size_t off = 0;
  for (int i = 0; i < n; i++) {
    const ctgpu_batch_problem& q = problems[i];
    BatchEntry& e = b->probs[i];
    if (!q.d_sino || !q.h_view_angles || !q.d_image)
      return fail(CTGPU_ERR_INVALID, "problem " + std::to_string(i) + ": null buffer");
    if (q.geometry.n_view < 1)
      return fail(CTGPU_ERR_INVALID, "problem " + std::to_string(i) + ": no views");
    int rc = ctgpu_recon_create(&q.geometry, q.nx, q.ny, q.filter_name, q.filter_param,
                                q.filter_method, q.zeropad, q.filter_generation, q.interp_name, 1,
                                q.backproj_name, nullptr, &e.plan);
    if (rc) return fail(rc, "problem " + std::to_string(i) + ": " + ctgpu_last_error());
    if (e.plan->bproj == kDiff || e.plan->bproj == kIDiff)
      return fail(CTGPU_ERR_UNSUPPORTED, "problem " + std::to_string(i) +
                                             ": diff / idiff backprojectors are not batched");
    if (q.sino_pitch < q.geometry.n_det) return fail(CTGPU_ERR_INVALID, "sino_pitch < n_det");
    e.d_sino = q.d_sino;
    e.sinoPitch = q.sino_pitch;
    e.d_image = q.d_image;
    const int nView = q.geometry.n_view;
    e.filtOff = off;
    off = align256(off + sizeof(float) * (size_t)nView * e.plan->pitch);
    e.angOff = off;
    off = align256(off + sizeof(double) * (size_t)nView);
    float scale = raw_scale(e.plan);
    if (e.plan->bproj != kTrig) scale = (float)(scale * e.plan->rotScale);   // PostProcessing
    // pointers into the arena are filled in below, once it exists
    e.L = make_launch(e.plan, nView, e.plan->pitch, nullptr, nullptr, e.d_image, 0, scale, 1, 0, 0);
    if (!table_prep_info(e.L, &e.prep))
      return fail(CTGPU_ERR_UNSUPPORTED, "problem " + std::to_string(i) +
                                             ": image pixels behind the fan-beam source");
    e.scratchOff = off;
    off = align256(off + e.prep.recBytes + e.prep.rowBytes);
  }
  b->arenaBytes = off;
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&b->d_arena), off));
  for (int i = 0; i < n; i++) {
    BatchEntry& e = b->probs[i];
    e.L.angles = reinterpret_cast<const double*>(b->d_arena + e.angOff);
    e.L.filtered = reinterpret_cast<const float*>(b->d_arena + e.filtOff);
    CUDA_TRY(cudaMemcpy(b->d_arena + e.angOff, problems[i].h_view_angles,
                        sizeof(double) * e.L.nViews, cudaMemcpyHostToDevice));
    const int tiles = ((e.L.nx + 31) / 32) * ((e.L.ny + 31) / 32);
    for (int t = 0; t < tiles; t++) b->items.push_back(BatchItem{i, t});
    // the (tile, view) records depend on the geometry, the image grid and the
    // view angles only, all fixed from here on: built once, kept in the arena
    CUDA_TRY(launch_tile_setup(e.L, b->d_arena + e.scratchOff, nullptr));
  }
  CUDA_TRY(cudaStreamSynchronize(nullptr));
  // longest first: a tile's cost is its problem's view count
  std::stable_sort(b->items.begin(), b->items.end(), [&](const BatchItem& x, const BatchItem& y) {
    return b->probs[x.problem].L.nViews > b->probs[y.problem].L.nViews;
  });
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&b->d_probs), sizeof(BatchProblem) * n));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&b->d_items), sizeof(BatchItem) * b->items.size()));
  CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&b->d_counter), sizeof(int)));
  CUDA_TRY(cudaMemcpy(b->d_items, b->items.data(), sizeof(BatchItem) * b->items.size(),
                      cudaMemcpyHostToDevice));
  for (int k = 0; k < kSideStreams; k++) {
    CUDA_TRY(cudaStreamCreateWithFlags(&b->side[k], cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
  }
  CUDA_TRY(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
  CUDA_TRY(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking));
  *out = b.release();
  return ok();
}

int ctgpu_batch_run(ctgpu_batch* b, void* stream) {
  if (!b) return fail(CTGPU_ERR_INVALID, "null batch");
  cudaStream_t s = (cudaStream_t)stream;
  if (b->exec) {
    CUDA_TRY(cudaGraphLaunch(b->exec, s));
    return ok();
  }
  int rc = batch_enqueue_prep(b, s);
  if (rc) return rc;
  if (!b->shaped) {
    rc = (b->flags & CTGPU_BATCH_AUTOTUNE) ? batch_tune(b, s) : batch_set_shape(b, b->shape);
    if (rc) return rc;
    b->shaped = true;
  }
  rc = batch_enqueue_backprojection(b, s);
  if (rc) return rc;
  if (b->flags & CTGPU_BATCH_GRAPH) {
    // record the same work on a private stream; later runs replay it
    CUDA_TRY(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal));
    rc = batch_enqueue_prep(b, b->capture);
    if (rc == CTGPU_OK) rc = batch_enqueue_backprojection(b, b->capture);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->capture, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    CUDA_TRY(e);
    b->graph = g;
    CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
  }
  return ok();
}

int ctgpu_batch_shape(const ctgpu_batch* b, int* blocksPerSM, int* viewsPerStage) {
  if (!b) return fail(CTGPU_ERR_INVALID, "null batch");
  if (blocksPerSM) *blocksPerSM = b->shape.blocksPerSM;
  if (viewsPerStage) *viewsPerStage = b->shape.cvCap;
  return ok();
}

void ctgpu_batch_destroy(ctgpu_batch* b) { delete b; }

}  // extern "C"
