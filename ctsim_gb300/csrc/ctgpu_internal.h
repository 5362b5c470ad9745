// ctgpu_internal.h -- structures shared by the host core and the sm_103a kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ctgpu {

// ----- constants of the reference (include/ctsupport.h:167-179) -----------
constexpr double kPi = 3.14159265358979323846;
constexpr double kHalfPi = 1.57079632679489661923;
constexpr double kTwoPi = 6.28318530717958647692;
constexpr double kSqrt2 = 1.414213562373095049;

enum ElemType { kRect = 1, kTriangle = 2, kEllipse = 3, kSector = 4, kSegment = 5 };
enum Geometry { kParallel = 0, kEquiangular = 1, kEquilinear = 2 };
enum Interp { kNearest = 0, kLinear = 1, kCubic = 2 };
enum Backproj { kTrig = 0, kTable = 1, kDiff = 2, kIDiff = 3 };

// One phantom element, FP64 (PhantomElement, libctsim/phantom.cpp:554-566).
struct PElem {
  int type;
  int pad;
  double cx, cy, u, v, rot, atten;
  double cosr, sinr;
  double bx0, by0, bx1, by1;   // outline-polygon bounding box
  // view-independent FP32 values of the ray-sum kernel, set with the box:
  // box centre minus element centre, box half sizes, circumscribed radius
  // (widened by its margin), inscribed radius less the margin
  float dcbx, dcby, hx, hy, rbox, rin;
  // ellipse chords: E = (ra/u)^2 + (rb/v)^2 of a unit direction (rx, ry) as
  // the quadratic form qa rx^2 + qb rx ry + qc ry^2, and u v (FP32 products
  // of the FP32 semi-axes); set by set_elem_quadratic
  float qa, qb, qc, uv;
};

// PElem's ellipse quadratic form from its semi-axes and rotation (FP64, then
// FP32): once per element, not per view
__host__ __device__ inline void set_elem_quadratic(PElem& e) {
  const double iu2 = 1.0 / (e.u * e.u), iv2 = 1.0 / (e.v * e.v);
  const double c = e.cosr, sn = e.sinr;
  e.qa = (float)(c * c * iu2 + sn * sn * iv2);
  e.qb = (float)(2.0 * c * sn * (iu2 - iv2));
  e.qc = (float)(sn * sn * iu2 + c * c * iv2);
  e.uv = (float)e.u * (float)e.v;
}

// Source / detector end points of one view after the reference's incremental
// rotation (libctsim/scanner.cpp:301-417), and its view angle.
struct ViewPos {
  double xs1, ys1, xs2, ys2, xd1, yd1, xd2, yd2, angle;
};

// Per-view ray geometry derived on the host in FP64 from a ViewPos (shared by
// every phantom scanned with the view), with the FP32 copies the rays use.
struct RayView {
  double S0x, S0y, dSx, dSy;       // source of detector 0 (parallel: per detector step)
  double D0x, D0y, dDx, dDy;       // detector point of ray 0 and per-ray step
  double alpha0, delta;            // equiangular arc: angle of ray 0, step
  double c0, s0, cm, sm;           // equiangular: cos/sin of alpha0 and of the arc's middle
  double midRel, invDelta;         // middle - alpha0, 1 / delta
  float rsx, rsy, stx, sty;        // FP32: D0 - S0, per-ray step
  float hdelta, ca0, sa0, Sx, Sy;  // FP32: delta / 2, cos/sin alpha0, source
  float cmf, smf, midRelf, invDeltaf;   // FP32: cm, sm, midRel, invDelta
};
RayView make_ray_view(int geometry, int nDet, int nSample, double angularDetLen,
                      double angularDetInc, const ViewPos& vp);

struct RaysumLaunch {
  int geometry, nDet, nSample, nElem, nViews, pitch, rowOffset;
  double centerDetectorLength, angularDetLen, angularDetInc;
  const PElem* elems;
  const RayView* views;   // nViews
  const float2* sdirs;    // parallel: [nViews][nSample] unit ray directions
  const double2* arc;     // equiangular: (cos, sin) of t * delta, t < nDet * nSample
  const float2* arcHalf;  // equiangular: (cos, sin) of t * delta / 2 (FP32)
  float* sino;
  unsigned int* status;
  // several phantoms, one sinogram each (grid.y): phantom z's elements are
  // elems[elemOffset[z] .. elemOffset[z+1]); nElem is then the largest count.
  // elemOffset null: one phantom of nElem elements.
  int nSlices;
  const int* elemOffset;
  size_t sliceStride;   // floats between the sinograms
  // one element list per view (3-D phantoms): view v's nElem elements start
  // at elems + v * nElem; an element of type < 0 is absent from that view
  int elemsPerView;
  // set by launch_raysum: views per ray block, 1 / centerDetectorLength, and
  // atan(j / 64) for j = 0..64 (the element records' table-driven arctangent)
  int viewsPerBlock;
  double invCD;
  double atan64[65];
};

// Filter: out[v][n] = sum_i (w[i] * in[v][i]) * taps[n - i + nDet - 1]
struct FilterLaunch {
  int nDet, nViews, inPitch, outPitch;
  int fftN;                 // circular convolution length (power of two >= 2*nDet-1)
  const float2* spectrum;   // fftN: DFT of the filter kernel / fftN
  const float2* twiddle;    // fftN: exp(-2 pi i m / fftN)
  const float* weights;     // nDet (fan pre-weighting, 1 for parallel)
  const float* in;          // [nBatch][nViews][inPitch]
  float* out;               // [nBatch][nViews][outPitch]
  int nBatch;
  size_t inSliceStride, outSliceStride;
  // a launch of few blocks may give each transform N / 8 threads (the
  // single-slice entry points; batched launches keep one arithmetic)
  int narrowOk;
  // optional: the table-family backprojection's interval rows of the filtered
  // views (k_backproject.cu's layout: kRowPad zero elements before sample 0,
  // rowsPitch elements per view, rowsSliceStride elements between slices),
  // written by the filter kernel from its output when rows != null and the
  // kernel chosen can (launch_filter reports it)
  void* rows;
  int rowsInterp;
  int rowsPitch;
  size_t rowsSliceStride;
};
// zero row elements before sample 0 of an interval row
constexpr int kRowPad = 4;

// Backprojection of one problem.
struct BackprojLaunch {
  int geometry, interp, bproj;
  int nDet, nx, ny, nViews, pitch;
  int iDetCenter;
  double detInc, xMin, yMin, xInc, yInc, focalLength, sdl, rotScale;
  double minSourceDist;   // fan beams: lower bound of the source-to-pixel distance
  const double* angles;   // device, nViews
  const float* filtered;  // device, [nBatch][nViews][pitch]
  float* image;           // device, [nBatch][nx][ny]
  int nBatch;             // slices sharing geometry and view angles (grid.z)
  size_t filtSliceStride, imageSliceStride;   // elements between slices
  int accumulate;         // add into image instead of overwriting
  float outScale;         // applied to this launch's contribution (rotScale for trig)
  unsigned int* status;
  // table family: the (tile, view) records in scratch were built by an earlier
  // launch of the same plan and view angles, ordered before this one
  int reuseRecords;
  // table family, one slice: > 1 splits its views into this many groups
  // (grid.z), each writing a partial image that one pass then sums in group
  // order (table_view_groups picks it); partial: the groups' images
  // [viewGroups][nx][ny] (set by the launch, in the set-up scratch)
  int viewGroups;
  float* partial;
  // table family: the interval rows in scratch were written by the filter
  // launch ordered before this one (launch_filter's rows)
  int rowsReady;
};

struct HelicalLaunch {
  int nDet, nViewIn, nViewOut, offsetView, pitch;
  double dbeta, dgamma, fan;
  // equilinear restatement: a detector's fan angle is atan(pos / sdl), pos
  // = (id - (nDet-1)/2) * dgamma (no reference counterpart)
  int equilinear;
  double sdl;
  const float* in;    // original data
  float* out;
  unsigned int* status;
};
constexpr unsigned int kStatusFeatherRange = 2u;

// One output sample's 180LI terms: own ray (same view and detector) with
// weight w0 when own != 0, complementary ray (view ivc >= 0, mirrored
// detector) with weight wc; views counted from the slice's first input view.
struct HelicalTap {
  double w0, wc;
  int own, ivc;
};
// HalfScanFeather of one output sample: the 180LI sample (v, d) times w;
// bad: the reference's "Shouldn't be here" case
struct FeatherTap {
  double w;
  int v, d, bad, pad;
};
struct HelicalSlicesLaunch {
  int nDet, nViewOut, nSlices, inPitch, outPitch, pad;
  const float* in;
  const int* offsets;          // device, nSlices: first input view of each slice
  const HelicalTap* interp;    // [nViewOut][nDet]
  const FeatherTap* feather;   // [nViewOut][nDet] or null
  double sf;                   // feathering's final scale nView * dbeta / pi
  float* out;                  // [nSlices] x outSliceStride
  size_t outSliceStride;
  unsigned int* status;
};
// Phantom::convertToImagefile on the device (k_raysum.cu)
struct RasterElem {
  double m[3][3];     // PhantomElement's phantom-to-object map (row vectors)
  double u, v, atten;
  int type, pad;
};
struct RasterLaunch {
  int nx, ny, nsample, nElem;
  const RasterElem* elems;   // list order
  const double* xcol;        // nx: each column's x, accumulated as the reference does
  const double* yrow;        // ny
  double kxinc, kyinc, kxofs, kyofs, factor;
  float* image;              // [nx][ny]
};
cudaError_t launch_raster(const RasterLaunch& L, cudaStream_t s);

// Projections::interpolateToParallel on the device (k_rebin.cu)
struct RebinLaunch {
  int nDet, nView, pitch, outPitch, sortN, pad;
  const float* in;          // [nView][pitch] fan-beam
  const double* angles;     // nView view angles
  const double* gam;        // nDet: fan angle of each detector
  const int* group;         // nDet: rank of the detector's t = FL sin(gamma)
  const double* thetaOut;   // nView output view angles
  const double* tSorted;    // nDet: t of each rank
  const double* posOut;     // nDet output detector positions
  float* tmp;               // [nView][nDet]
  float* out;               // [nView][outPitch]
};
cudaError_t launch_rebin(RebinLaunch L, cudaStream_t s);
size_t rebin_sort_bytes(int nView);

cudaError_t launch_helical_tables(const HelicalLaunch& L, const double* gammaTab,
                                  HelicalTap* interp, FeatherTap* feather, cudaStream_t s);
cudaError_t launch_helical_slices(const HelicalSlicesLaunch& L, cudaStream_t s);

// status bits written by kernels
constexpr unsigned int kStatusTimeout = 1u;

// the C ABI's per-thread last-error message (ctgpu_api.cpp)
void set_last_error(const char* msg);

// device status word (k_common.cu)
unsigned int* status_pointer();
cudaError_t status_read_and_clear(unsigned int* value);

// kernel entry wrappers (defined in the .cu files)
cudaError_t launch_raysum(const RaysumLaunch& L, cudaStream_t s);
// Per-view cross-sections of ellipsoids: base[k] is ellipsoid k as a 2-D
// ellipse at its full semi-axes, zc[k] its (z centre, z semi-axis); out[v][k]
// is the ellipse cut at z0 + v dz, scaled about its centre, or absent.
cudaError_t launch_ellipsoid_sections(const PElem* base, const double2* zc, int n, int nViews,
                                      double z0, double dz, PElem* out, cudaStream_t s);
// d(sum_{v,d} gsino[v][d] sino[v][d]) / d(cx, cy, u, v, theta, atten) of every
// element (ellipses) into grad[6 * nElem] (FP64, accumulated: zero it first)
cudaError_t launch_raysum_ellipse_grad(const RaysumLaunch& L, const float* gsino, double* grad,
                                       cudaStream_t s);
// Many scans (each its own geometry, detectors, views and phantom) in one
// ray launch.  raysum_prepare completes a descriptor (views per block, 1/CD,
// the arctangent table) and returns its ray blocks' shared memory.  d_probs:
// the n descriptors in device memory; d_rayStart: n + 1 block offsets (a
// problem has ceil(nViews / viewsPerBlock) blocks).
size_t raysum_prepare(RaysumLaunch& L);
cudaError_t launch_raysum_multi(const RaysumLaunch* d_probs, const int* d_rayStart,
                                int rayBlocks, int n, size_t smem, cudaStream_t s);
cudaError_t launch_unit_pulse(float* sino, int nViews, int nDet, int pitch, int rowOffset,
                              cudaStream_t s);
// *rowsWritten (if given): whether the launch also wrote L.rows
cudaError_t launch_filter(const FilterLaunch& L, cudaStream_t s, bool* rowsWritten = nullptr);
size_t backproject_scratch_bytes(const BackprojLaunch& L);
// blocks of the table-family main kernel resident per SM (its occupancy target)
int backproject_table_ctas_per_sm();
// view groups for a one-slice table-family launch on `sms` SMs (1: no split)
int table_view_groups(const BackprojLaunch& L, int sms);
constexpr int kBackprojTile = 32;   // image pixels per tile side

// The table-family backprojection as set-up launches plus a main launch, for
// the batched path (many problems of different sizes, one persistent launch).
// Equiangular fan beams: the arctangent series' coefficients of z^3, z^5 and
// z^7 times the detector scale c5 = 1/detInc (the records' c[5]), so that a
// pixel's position is one Horner chain in z^2:
//   q = f + z*(c5 + z^2*(a3 + z^2*(a5 + z^2*a7)))
struct FanSeries {
  float a3, a5, a7;
};
struct TablePrep {
  int kind;        // main-kernel variant: geometry, interpolation, arctangent
  int win;         // row elements staged per (tile, view)
  int rpitch;      // row elements per view
  int elemBytes;   // bytes per row element (4, 8 or 16)
  float eps;       // FP32 position margin around jumps of the result
  FanSeries fan;   // equiangular: the scaled series coefficients
  size_t recBytes, rowBytes;   // scratch: the records, then the rows
};
bool table_prep_info(const BackprojLaunch& L, TablePrep* out);
// where a table-family launch keeps its interval rows in scratch: byte offset,
// elements per view and the interpolation; false for other backprojectors
bool table_rows_layout(const BackprojLaunch& L, size_t* offsetBytes, int* rpitch, int* interp);
// interval rows and (tile, view) records of one problem into scratch
cudaError_t launch_table_prep(const BackprojLaunch& L, const TablePrep& P, void* scratch,
                              cudaStream_t s);
// the (tile, view) records alone (geometry and view angles only)
cudaError_t launch_tile_setup(const BackprojLaunch& L, void* scratch, cudaStream_t s);

struct BatchProblem {
  BackprojLaunch L;   // one slice: nBatch 1
  const void* recs;
  const void* rows;
  int kind, win, rpitch, elemBytes, cv, tilesX;
  float eps;
  FanSeries fan;
};
struct BatchItem { int problem, tile; };
struct BatchShape { int blocksPerSM, cvCap; };
// views per pipeline stage of a problem under a launch shape (0: does not fit)
int batch_views_per_stage(const TablePrep& P, const BatchShape& shape);
// kernel attributes for a shape; call before capturing a launch in a graph
cudaError_t prepare_backproject_batch(const BatchShape& shape, int* gridBlocks);
// d_counter: one int, zero at launch (the work-queue head)
cudaError_t launch_backproject_batch(const BatchProblem* d_probs, const BatchItem* d_items,
                                     int nItems, int* d_counter, const BatchShape& shape,
                                     int gridBlocks, unsigned int* status, cudaStream_t s);
cudaError_t launch_backproject_views(const BackprojLaunch& L, const void* views, void* scratch,
                                     cudaStream_t s);
cudaError_t launch_scale_image(float* image, size_t n, float scale, cudaStream_t s);
cudaError_t launch_project_table(const BackprojLaunch& L, const float* image, float* sino,
                                 float scale, cudaStream_t s);
cudaError_t launch_helical180li(const HelicalLaunch& L, cudaStream_t s);
cudaError_t launch_halfscan_feather(const HelicalLaunch& L, cudaStream_t s);

// ----- file formats and image utilities (k_fileio.cu) ----------------------
// .pj view records: f64 angle, u32 nDet, nDet x f32, as 3 + nDet 32-bit words
cudaError_t launch_pj_pack(const float* sino, int pitch, const double* angles, int nViews,
                           int nDet, uint32_t* out, cudaStream_t s);
// status[0] += records whose nDet word differs from nDet, status[1] = min view
cudaError_t launch_pj_unpack(const uint32_t* in, int nViews, int nDet, float* sino, int pitch,
                             double* angles, int viewOffset, unsigned int* status,
                             cudaStream_t s);
// pj2if: image[ix][iy] (nDet x nView, column-major) = sino[nView - 1 - iy][ix]
cudaError_t launch_sino_to_image(const float* sino, int pitch, int nView, int nDet, float* image,
                                 cudaStream_t s);
cudaError_t launch_f64_to_f32(const double* in, float* out, size_t n, cudaStream_t s);
// op 0 add, 1 subtract, 2 multiply, 3 divide (FP32)
cudaError_t launch_image_arith(int op, const float* a, const float* b, float* out, size_t n,
                               cudaStream_t s);
// comparative statistics of image pairs (nx * ny < 2^31): part holds nImages x
// compare_blocks(nx, ny) x kCmpParts float pairs, out nImages x (d, r, e)
constexpr int kCmpParts = 7;
struct CompareLaunch {
  const float* a;
  const float* b;
  size_t strideA, strideB;   // floats between images
  int nx, ny, nImages;
  float2* part;
  double* out;
};
int compare_blocks(int nx, int ny);
cudaError_t launch_image_compare(const CompareLaunch& L, cudaStream_t s);

// ----- polar and direct-Fourier images (k_fourier.cu) ----------------------
struct PolarLaunch {
  int nx, ny, cols;            // columns >= cols are zeroed
  const double* xs;            // [nx] pixel-centre x, accumulated as the reference does
  const double* ys;            // [ny]
  double rotInc, rotStart, detInc, detCenter;
  const float* data;           // [nView][pitch] real rows, or float2 [nView][pitch]
  int complexData, pitch, nView, nPos;
  int interp;                  // 0 nearest, 1 bilinear
  float* outRe;
  float* outIm;                // may be null
};
cudaError_t launch_polar(const PolarLaunch& L, cudaStream_t s);

struct FourierViewsLaunch {
  const float* sino;           // parallel rows [nView][pitch]
  int pitch, nView, nDet;
  int nInterp, N, iMid;        // points interpolated, transform length, insertion point
  const double* posTable;      // [nInterp] detector positions of the interpolated points
  double projScale, fftScale;
  const float2* twiddle;       // [N] exp(-2 pi i m / N)
  float2* spec;                // [nView][N] out, natural order
};
cudaError_t launch_fourier_views(const FourierViewsLaunch& L, cudaStream_t s);

struct IfftLaunch {
  int nx, ny;
  const float* inRe;           // [nx][ny]
  const float* inIm;
  float2* tmp;                 // [nx][ny] scratch
  const float2* twX;           // [nx] exp(-2 pi i m / nx)
  const float2* twY;           // [ny]
  float* out;                  // [nx][ny] magnitude, natural order
};
cudaError_t launch_ifft_magnitude(const IfftLaunch& L, cudaStream_t s);
size_t line_smem_bytes(int n);

}  // namespace ctgpu
