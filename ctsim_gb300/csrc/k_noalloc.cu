// k_noalloc.cu -- the "diff" backprojection with its scratch in a fixed,
// file-scope device array, for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: plug-ins hosted by an
// application that owns every device allocation (its own allocator or a fixed
// memory budget), and real-time loops that must not block on the allocator.
// ctgpu_backproject_diff_noalloc() serves them: the caller passes the filtered
// sinogram and the image; the per-view steps and the per-(view, column) row
// ranges the diff backprojector needs live in g_noalloc_scratch below.
//
// The array is static device memory of kNoAllocScratchBytes (16 MiB): every
// GPU that loads the library keeps it until the process exits.  Its device
// address is looked up once per device, on that device's first call (see the
// entry point's comment in include/ctgpu.h).  All calls share the array and it
// keeps the last call's contents; each call writes every element it later
// reads (the view records by a small kernel whose parameters carry them, the
// row ranges by the set-up kernel), so nothing needs clearing.  Calls that
// overlap on the GPU (different streams or threads) race on the array.
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <strings.h>

#include "../../include/ctgpu.h"
#include "ctgpu_internal.h"

namespace ctgpu {
struct DiffViewRecord { double dx, dy, colStart; };   // layout of k_backproject.cu's DiffView
struct DiffColRecord { double c0; int a, b; };        // layout of k_backproject.cu's DiffCol

// Up to kViewsPerParamBlock view records travel by value as one kernel's
// parameters (3 KB of the 4 KB parameter space), so no host buffer is read
// after the launch call returns and no host-to-device copy is queued.
constexpr int kViewsPerParamBlock = 128;
struct DiffViewParams { DiffViewRecord r[kViewsPerParamBlock]; };

__global__ void noalloc_store_views_kernel(DiffViewParams p, int n, DiffViewRecord* dst) {
  int i = threadIdx.x;
  if (i < n) dst[i] = p.r[i];
}
}  // namespace ctgpu

using namespace ctgpu;

namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

int fail(int code, const std::string& msg) {
  set_last_error(msg.c_str());
  return code;
}

// Device address of g_noalloc_scratch on the current device, looked up once per
// device with that device current.  Host code must not use the symbol itself:
// on the host it is only a stand-in, not a device address.
// Concurrent first calls from several host threads may both look the address
// up; they store the same value, and the atomics make that well defined.
cudaError_t scratch_address(unsigned char** out) {
  static std::atomic<unsigned char*> ptrs[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  unsigned char* ptr = ptrs[dev].load(std::memory_order_acquire);
  if (!ptr) {
    e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    ptrs[dev].store(ptr, std::memory_order_release);
  }
  *out = ptr;
  return cudaSuccess;
}

}  // namespace

extern "C" int ctgpu_backproject_diff_noalloc(const ctgpu_geometry* g, int nx, int ny,
                                              const char* interp_name, const ctgpu_roi* roi,
                                              const float* d_filtered, int filtered_pitch,
                                              const double* h_view_angles, int n_views,
                                              float* d_image, int flags, void* stream) {
  if (!g || !interp_name || !d_filtered || !h_view_angles || !d_image)
    return fail(CTGPU_ERR_INVALID, "null argument");
  if (g->geometry != kParallel)
    return fail(CTGPU_ERR_INVALID, "the diff backprojector is a parallel-geometry method");
  int interp = !strcasecmp(interp_name, "nearest") ? kNearest
               : !strcasecmp(interp_name, "linear") ? kLinear
               : !strcasecmp(interp_name, "cubic") ? kCubic : -1;
  if (interp < 0) return fail(CTGPU_ERR_INVALID, std::string("Invalid interpolation name ") + interp_name);
  if (nx < 1 || ny < 1 || g->n_det < 2 || n_views < 0 || filtered_pitch < g->n_det)
    return fail(CTGPU_ERR_INVALID, "bad sizes");
  const size_t viewBytes = sizeof(DiffViewRecord) * (size_t)n_views;
  const size_t colOffset = (viewBytes + 255) & ~(size_t)255;
  const size_t need = colOffset + sizeof(DiffColRecord) * (size_t)n_views * (size_t)nx;
  if (need > kNoAllocScratchBytes)
    return fail(CTGPU_ERR_INVALID,
                "n_views * nx too large for the fixed 16 MiB scratch: needs " +
                    std::to_string(need) + " bytes (at most about " +
                    std::to_string(kNoAllocScratchBytes / 16) + " view-columns)");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* scratch = nullptr;
  cudaError_t e = scratch_address(&scratch);
  if (e != cudaSuccess) return fail(CTGPU_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));

  // Backproject::Backproject (libctsim/backprojectors.cpp:264-319)
  const int nDet = g->n_det, iDetCenter = (nDet - 1) / 2;
  const double rotScale = kPi / g->n_view;
  double phmLen = g->view_diameter / kSqrt2;
  double xMin = -phmLen / 2, xMax = xMin + phmLen, yMin = -phmLen / 2, yMax = yMin + phmLen;
  if (roi) {
    if (roi->x_min > xMin) xMin = roi->x_min;
    if (roi->x_max < xMax) xMax = roi->x_max;
    if (roi->y_min > yMin) yMin = roi->y_min;
    if (roi->y_max < yMax) yMax = roi->y_max;
    if (xMin > xMax) std::swap(xMin, xMax);
    if (yMin > yMax) std::swap(yMin, yMax);
  }
  const double xInc = (xMax - xMin) / nx, yInc = (yMax - yMin) / ny;
  const double x0 = xMin + xInc / 2, y0 = yMin + yInc / 2;
  const double startR = std::sqrt(x0 * x0 + y0 * y0), startPhi = std::atan2(y0, x0);

  // per-view steps (BackprojectDiff::BackprojectView, backprojectors.cpp:522-527),
  // computed on the host in FP64 like the allocating path's, and stored into
  // the scratch array by kernels that receive them as parameters
  DiffViewParams blk;
  for (int v0 = 0; v0 < n_views; v0 += kViewsPerParamBlock) {
    int nv = n_views - v0 < kViewsPerParamBlock ? n_views - v0 : kViewsPerParamBlock;
    for (int i = 0; i < nv; i++) {
      double th = h_view_angles[v0 + i];
      blk.r[i].dx = xInc * std::cos(th) / g->det_inc;
      blk.r[i].dy = yInc * std::sin(th) / g->det_inc;
      blk.r[i].colStart = iDetCenter + startR * std::cos(th - startPhi) / g->det_inc;
    }
    noalloc_store_views_kernel<<<1, kViewsPerParamBlock, 0, st>>>(
        blk, nv, (DiffViewRecord*)scratch + v0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CTGPU_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  }
  BackprojLaunch L{};
  L.geometry = kParallel;
  L.interp = interp;
  L.bproj = kDiff;
  L.nDet = nDet;
  L.nx = nx;
  L.ny = ny;
  L.nViews = n_views;
  L.pitch = filtered_pitch;
  L.iDetCenter = iDetCenter;
  L.detInc = g->det_inc;
  L.xMin = xMin;
  L.yMin = yMin;
  L.xInc = xInc;
  L.yInc = yInc;
  L.rotScale = rotScale;
  L.filtered = d_filtered;
  L.image = d_image;
  L.nBatch = 1;
  L.accumulate = (flags & CTGPU_RUN_ACCUMULATE) ? 1 : 0;
  L.outScale = (flags & CTGPU_RUN_POSTPROCESS) ? (float)rotScale : 1.f;
  if (n_views == 0) {
    if (!L.accumulate) {
      e = cudaMemsetAsync(d_image, 0, sizeof(float) * (size_t)nx * ny, st);
      if (e != cudaSuccess) return fail(CTGPU_ERR_CUDA, cudaGetErrorString(e));
    }
    set_last_error("");
    return CTGPU_OK;
  }
  e = launch_backproject_views(L, scratch, scratch + colOffset, st);
  if (e != cudaSuccess) return fail(CTGPU_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  set_last_error("");
  return CTGPU_OK;
}
