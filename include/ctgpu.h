/* ctgpu.h -- C ABI of the GB300 simulate-and-reconstruct library (libctgpu.so).
 *
 * Drop-in boundary for CTSim's hot path: analytic phantom ray-sums
 * (Scanner::collectProjections), projection filtering (ProcessSignal) and
 * backprojection (Backprojector) as driven by Reconstructor, plus the helical
 * 180LI / half-scan pre-step.  Every entry point below names the CTSim 5.2.0
 * interface (file:line) whose behaviour it reproduces.  Plain C types only:
 * pointers, sizes, doubles; no C++ or torch types cross this boundary.
 *
 * Conventions
 *   - Return value: CTGPU_OK (0) or one of the CTGPU_ERR_* codes; the message
 *     of the last failure on the calling thread is ctgpu_last_error().
 *   - Names (geometry, filter, method, generation, interpolation,
 *     backprojector) use the reference's case-insensitive name tables,
 *     including its quirks ("shepp" selects the |w|*sinc response and
 *     "abs_sinc" the Shepp response; the method "fouier-table" is spelt as in
 *     the reference).
 *   - d_ prefix: device pointer (cudaMalloc'ed or equivalent); h_ prefix: host
 *     pointer.  Sinograms are row-major [view][detector] FP32 with a row pitch
 *     in floats (>= n_det; a multiple of 4 keeps rows 16-byte aligned for the
 *     bulk copies the backprojector issues).  Images are column-major
 *     [ix][iy] FP32 like CTSim's ImageFile (v[ix][iy]).
 *   - `stream` is a cudaStream_t passed as void* (NULL = default stream).
 *     Calls taking a stream only enqueue work; ctgpu_sync() waits and reports
 *     device-side failures (a bounded wait that gave up).
 *   - Handles are not thread-safe; use one per thread, like the reference's
 *     one-Reconstructor-per-thread model (src/threadrecon.cpp:219-255).
 */
#ifndef CTGPU_H
#define CTGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CTGPU_ABI_VERSION 1

enum {
  CTGPU_OK = 0,
  CTGPU_ERR_INVALID = 1,      /* bad argument / name; the reference's fail() + failMessage() */
  CTGPU_ERR_UNSUPPORTED = 2,  /* valid request the library does not implement */
  CTGPU_ERR_CUDA = 3,         /* CUDA runtime error */
  CTGPU_ERR_NOMEM = 4,        /* allocation failure */
  CTGPU_ERR_TIMEOUT = 5,      /* a kernel's bounded wait gave up (see ctgpu_sync) */
  CTGPU_ERR_IO = 6            /* file could not be read */
};

/* geometry ids: libctsim/scanner.cpp:29-33 */
enum { CTGPU_GEOMETRY_PARALLEL = 0, CTGPU_GEOMETRY_EQUIANGULAR = 1, CTGPU_GEOMETRY_EQUILINEAR = 2 };

/* Message for the last non-OK return on this thread ("" if none). */
const char* ctgpu_last_error(void);
int ctgpu_abi_version(void);

/* Waits for `stream` and reports CTGPU_ERR_TIMEOUT if a kernel's bounded
 * shared-memory pipeline wait expired since the last call (the kernel then
 * stopped early and its output is invalid), CTGPU_ERR_CUDA on a CUDA error. */
int ctgpu_sync(void* stream);

/* ------------------------------------------------------------------------ */
/* Phantom -- replaces Phantom / PhantomElement (libctsim/phantom.cpp:58-256, */
/* :554-756).  Elements keep the reference's list order (last added first)   */
/* and the 360-point outline bounding box used to pre-reject rays.           */
/* ------------------------------------------------------------------------ */
typedef struct ctgpu_phantom ctgpu_phantom;

/* Phantom::Phantom() -- empty phantom */
int ctgpu_phantom_create(ctgpu_phantom** out);
/* Phantom::createFromPhantom (phantom.cpp:128-170): "herman", "shepp-logan", "unit-pulse" */
int ctgpu_phantom_create_builtin(const char* name, ctgpu_phantom** out);
/* Phantom::addPElem (phantom.cpp:237-256); type: rectangle|triangle|ellipse|sector|segment */
int ctgpu_phantom_add_element(ctgpu_phantom* p, const char* type, double cx, double cy, double u,
                              double v, double rot_deg, double atten);
/* Phantom::createFromFile (phantom.cpp:184-213): lines "type cx cy u v rot atten" */
int ctgpu_phantom_read_file(ctgpu_phantom* p, const char* filename);
/* xmin, xmax, ymin, ymax of the union of element bounding boxes (phantom.cpp:250-253) */
int ctgpu_phantom_bounds(const ctgpu_phantom* p, double bounds[4], int* n_elements);
/* Phantom::convertToImagefile (phantom.cpp:462-542), what phm2if does: each
 * pixel of d_image [nx][ny] (column-major, FP32 as ImageFile) is the mean
 * over nsample x nsample points of the summed attenuation of the elements
 * containing the point; extent (xmin, xmax, ymin, ymax) and increment
 * receive the image axes.  Images smaller than 2 x 2 are left untouched. */
int ctgpu_phantom_rasterize(const ctgpu_phantom* p, int nx, int ny, double view_ratio,
                            int nsample, float* d_image, double extent[4], double increment[2],
                            void* stream);
void ctgpu_phantom_destroy(ctgpu_phantom* p);

/* ------------------------------------------------------------------------ */
/* Scan geometry: the fields of a .pj header (libctsim/projections.cpp:485-546) */
/* ------------------------------------------------------------------------ */
typedef struct {
  int32_t geometry;           /* CTGPU_GEOMETRY_* */
  int32_t n_det;
  int32_t n_view;
  int32_t reserved;
  double rot_start, rot_inc;
  double det_start, det_inc;
  double view_diameter, focal_length, source_detector_length, fan_beam_angle;
} ctgpu_geometry;

/* ------------------------------------------------------------------------ */
/* Scanner -- replaces Scanner::Scanner (libctsim/scanner.cpp:86-224) and   */
/* Scanner::collectProjections (:280-533)                                    */
/* ------------------------------------------------------------------------ */
typedef struct ctgpu_scanner ctgpu_scanner;

/* Scanner::Scanner: rot_angle in radians (phm2pj passes fraction * 2*pi),
 * ratios as in tools/phm2pj.cpp (defaults 2, 2, 1, 1).  A scanner does not
 * change after create; it keeps the ray geometry of the last view range it
 * scanned in device memory (about 200 B per view) and rebuilds it only for
 * another range. */
int ctgpu_scanner_create(const ctgpu_phantom* p, const char* geometry_name, int n_det, int n_view,
                         int offset_view, int n_sample, double rot_angle,
                         double focal_length_ratio, double center_detector_ratio,
                         double view_ratio, double scan_ratio, ctgpu_scanner** out);
/* Projections::initFromScanner (projections.cpp:145-161) */
int ctgpu_scanner_geometry(const ctgpu_scanner* s, ctgpu_geometry* out);
/* Scanner::collectProjections(proj, phm, iStartView, iNumViews, iOffsetView,
 * iStorageOffset) (scanner.cpp:295-419): ray-sums of views
 * [start_view, start_view + n_views) into rows storage_offset.. of d_sino;
 * the view angles (FP64, accumulated exactly as the reference) go to
 * h_view_angles[storage_offset..] when non-NULL. */
int ctgpu_collect_projections(ctgpu_scanner* s, const ctgpu_phantom* p, int start_view,
                              int n_views, int offset_view, int storage_offset, float* d_sino,
                              int sino_pitch, double* h_view_angles, void* stream);
/* Same with a host sinogram [n_view][n_det]; copies in the call, synchronous. */
int ctgpu_collect_projections_host(ctgpu_scanner* s, const ctgpu_phantom* p, int start_view,
                                   int n_views, int offset_view, int storage_offset,
                                   float* h_sino, double* h_view_angles);
/* collectProjections of all n_view views for n_phantoms phantoms at once (one
 * launch): sinogram z at d_sinos + z * sino_slice_stride floats.  No
 * reference counterpart as one call (the reference scans one phantom per
 * Scanner::collectProjections).  Unit-pulse phantoms are not batched. */
int ctgpu_collect_projections_batch(ctgpu_scanner* s, const ctgpu_phantom* const* phantoms,
                                    int n_phantoms, float* d_sinos, int sino_pitch,
                                    long long sino_slice_stride, double* h_view_angles,
                                    void* stream);
/* Many scans of uneven shapes in one ray launch: problem
 * k scans phantoms[k] with scanners[k] (each its own geometry, nDet, nView
 * and nSample) over all its views into d_sinos[k] (rows of sino_pitches[k]
 * floats) and, if h_view_angles and h_view_angles[k] are not NULL, stores its
 * view angles there.  Each sinogram is what ctgpu_collect_projections writes
 * for the problem alone.  No reference counterpart as one call: the reference
 * scans one phantom per Scanner::collectProjections
 * (libctsim/scanner.cpp:280-419).  The scanners[0]'s staging and record
 * buffers carry the launch; unit-pulse phantoms are not batched. */
int ctgpu_collect_projections_multi(ctgpu_scanner* const* scanners,
                                    const ctgpu_phantom* const* phantoms, int n,
                                    float* const* d_sinos, const int* sino_pitches,
                                    double* const* h_view_angles, void* stream);
/* Helical scan of a 3-D phantom of n_ellipsoids ellipsoids, all n_view views
 * of the scanner (its geometry is that of a 2-D phantom; make it from the
 * ellipsoids' largest cross-sections).  View v sees the phantom's
 * cross-section at z = z0 + v * dz_per_view: ellipsoid k, ellipsoids[8k..8k+7]
 * = cx, cy, cz, a, b, c, rotation about z (degrees), attenuation, contributes
 * the ellipse (cx, cy, a s, b s) with s = sqrt(1 - ((z - cz)/c)^2) while
 * |z - cz| < c.  No reference counterpart (CTSim's phantoms are 2-D); the
 * views are projected as Scanner::projectSingleView does
 * (scanner.cpp:445-533). */
int ctgpu_collect_projections_ellipsoids(ctgpu_scanner* s, const double* ellipsoids,
                                         int n_ellipsoids, double z0, double dz_per_view,
                                         float* d_sino, int sino_pitch, double* h_view_angles,
                                         void* stream);
/* Gradient of the ray-sums of all n_view views with respect to the phantom's
 * ellipse parameters: h_grad[6 j + m] = sum over views v and detectors d of
 * d_grad_sino[v][d] * d sino[v][d] / d param_m of the j-th element added,
 * params (cx, cy, u, v, rot_deg, atten) as ctgpu_phantom_add_element.  Every
 * element must be an ellipse; the outline-box pre-rejection is held fixed
 * (it changes no chord but at tangency).  Synchronous.  No reference
 * counterpart (CTSim computes no derivatives). */
int ctgpu_raysum_ellipse_gradient(ctgpu_scanner* s, const ctgpu_phantom* p,
                                  const float* d_grad_sino, int sino_pitch, double* h_grad,
                                  void* stream);
void ctgpu_scanner_destroy(ctgpu_scanner* s);

/* ------------------------------------------------------------------------ */
/* Reconstruction -- replaces Reconstructor (libctsim/reconstruct.cpp:50-239) */
/* with its ProcessSignal (procsignal.cpp:82-629) and Backprojector          */
/* (backprojectors.cpp:100-743)                                              */
/* ------------------------------------------------------------------------ */
typedef struct ctgpu_recon ctgpu_recon;
typedef struct { double x_min, y_min, x_max, y_max; } ctgpu_roi;   /* ReconstructionROI */

/* Reconstructor::Reconstructor: filter bandwidth 1/det_inc and domain "spatial"
 * as the reference passes them.  interp_factor (preinterpolation) is accepted
 * for the convolution and O(n^2) Fourier methods, where the reference ignores
 * it, and rejected (CTGPU_ERR_UNSUPPORTED) for "fft", whose FFTW-only
 * preinterpolated output has no reference to match. */
int ctgpu_recon_create(const ctgpu_geometry* g, int nx, int ny, const char* filter_name,
                       double filter_param, const char* filter_method, int zeropad,
                       const char* filter_generation, const char* interp_name,
                       int interp_factor, const char* backproj_name, const ctgpu_roi* roi,
                       ctgpu_recon** out);
/* image axis extent and increments (Backproject::Backproject, backprojectors.cpp:284-315) */
int ctgpu_recon_image_axes(const ctgpu_recon* r, double extent[4], double increment[2]);
/* ProcessSignal::filterSignal for n_views rows (procsignal.cpp:543-629) */
int ctgpu_recon_filter(ctgpu_recon* r, const float* d_sino, int sino_pitch, int n_views,
                       float* d_filtered, int filtered_pitch, void* stream);
/* Backprojector::BackprojectView for n_views filtered rows with their view
 * angles; accumulate=0 clears d_image first (Backproject ctor's
 * arrayDataClear), 1 adds to it. */
int ctgpu_recon_backproject(ctgpu_recon* r, const float* d_filtered, int filtered_pitch,
                            const double* h_view_angles, int n_views, float* d_image,
                            int accumulate, void* stream);
/* Backprojector::PostProcessing (backprojectors.cpp:324-336, :435-442) */
int ctgpu_recon_postprocess(ctgpu_recon* r, float* d_image, void* stream);
/* Reconstructor::reconstructView(start, count) (+ postProcessing when
 * CTGPU_RUN_POSTPROCESS is set, i.e. reconstructAllViews). d_sino holds all
 * n_view rows; h_view_angles all n_view angles.  One slice fills few blocks,
 * so this call (and ctgpu_recon_run_host, ctgpu_recon_backproject) may split
 * the views into groups whose partial images are summed in a fixed order, and
 * filter with another transform split: its image equals the batched entry
 * points' to FP32 rounding (deterministic from call to call). */
#define CTGPU_RUN_POSTPROCESS 1
#define CTGPU_RUN_ACCUMULATE 2
int ctgpu_recon_run(ctgpu_recon* r, const float* d_sino, int sino_pitch,
                    const double* h_view_angles, int start_view, int n_views, float* d_image,
                    int flags, void* stream);
/* Reconstructor::reconstructAllViews with host buffers: h_sino [n_view][n_det],
 * h_image [nx][ny]; copies inside the call; synchronous. */
int ctgpu_recon_run_host(ctgpu_recon* r, const float* h_sino, const double* h_view_angles,
                         float* h_image);
/* Many slices of the same geometry and view angles in one launch per stage
 * (the batched form of reconstructAllViews): d_sinos holds n_batch sinograms
 * [n_view][sino_pitch] sino_slice_stride floats apart, d_images n_batch
 * images [nx][ny] image_slice_stride floats apart; flags as ctgpu_recon_run
 * (CTGPU_RUN_ACCUMULATE not supported). */
int ctgpu_recon_run_batch(ctgpu_recon* r, int n_batch, const float* d_sinos, int sino_pitch,
                          long long sino_slice_stride, const double* h_view_angles,
                          float* d_images, long long image_slice_stride, int flags,
                          void* stream);
/* ctgpu_recon_run_batch with host buffers: h_sinos n_batch sinograms
 * [n_view][n_det] back to back, h_images n_batch images [nx][ny] back to back.
 * Slices move in chunks through two sets of device buffers on two compute
 * streams, so the copies of one chunk overlap the reconstruction of its
 * neighbours and consecutive chunks overlap on the device (page-locked host
 * buffers make the copies asynchronous; pageable ones work, with less
 * overlap).  The chunk sizes (ctgpu_recon_host_chunks) keep the first and last
 * chunks' copies short; each buffer set builds its (tile, view) records once
 * per call.  Synchronous:
 * returns when h_images is written.  No reference counterpart (CTSim
 * reconstructs one slice per Reconstructor). */
int ctgpu_recon_run_batch_host(ctgpu_recon* r, int n_batch, const float* h_sinos,
                               const double* h_view_angles, float* h_images, int flags);
/* The chunk sizes ctgpu_recon_run_batch_host uses for n_batch slices on the
 * current device: the first min(count, max_sizes) go to sizes; returns the
 * number of chunks (>= 1), or a negative error.  No reference counterpart. */
int ctgpu_recon_host_chunks(const ctgpu_recon* r, int n_batch, int* sizes, int max_sizes);
/* Fixes ctgpu_recon_run_batch_host's chunk sizes: sizes[0..n) in turn from the
 * first slice (repeated, the last chunk cut short); n = 0 restores the planned
 * sizes.  No reference counterpart. */
int ctgpu_recon_set_host_chunks(ctgpu_recon* r, const int* sizes, int n);
/* Backprojection of n_batch filtered sinograms (same geometry and angles) in
 * one launch; flags: CTGPU_RUN_POSTPROCESS folds PostProcessing in. */
int ctgpu_recon_backproject_batch(ctgpu_recon* r, int n_batch, const float* d_filtered,
                                  int filtered_pitch, long long filtered_slice_stride,
                                  const double* h_view_angles, int n_views, float* d_images,
                                  long long image_slice_stride, int flags, void* stream);
/* Forward projection of a pixel image: the exact transpose of the parallel
 * table backprojector with linear interpolation (backprojectors.cpp:444-481)
 * without its rotScale, times `scale`:
 *   d_sino[v][d] = scale * sum_pixels image * w(pixel, view v, detector d).
 * Parallel geometry, plans made with backproj "table" and interp "linear". */
int ctgpu_recon_project(ctgpu_recon* r, const float* d_image, const double* h_view_angles,
                        int n_views, float* d_sino, int sino_pitch, float scale, void* stream);
void ctgpu_recon_destroy(ctgpu_recon* r);

/* ------------------------------------------------------------------------ */
/* Batched reconstruction of many problems of uneven sizes.  No reference   */
/* counterpart as one call: it is the reference's Reconstructor +           */
/* reconstructAllViews (reconstruct.cpp:50-239) for each problem, with the  */
/* problems' backprojections sharing one persistent launch.                 */
/* ------------------------------------------------------------------------ */
typedef struct ctgpu_batch ctgpu_batch;
typedef struct {
  ctgpu_geometry geometry;          /* the problem's scan (.pj header fields) */
  int nx, ny;                       /* image size */
  const char* filter_name;          /* as ctgpu_recon_create */
  double filter_param;
  const char* filter_method;
  int zeropad;
  const char* filter_generation;
  const char* interp_name;          /* nearest, linear, cubic */
  const char* backproj_name;        /* table or trig (parallel); fan beams use their own */
  const float* d_sino;              /* device [n_view][sino_pitch], read at every run */
  int sino_pitch;
  const double* h_view_angles;      /* n_view angles, copied at create */
  float* d_image;                   /* device [nx][ny], written at every run */
} ctgpu_batch_problem;
#define CTGPU_BATCH_AUTOTUNE 1   /* time the launch shapes on the first run, keep the fastest */
#define CTGPU_BATCH_GRAPH 2      /* capture the batch in a CUDA graph after the first run, replay it */
/* Plans every problem (filters, windows, work list) and builds its
 * backprojection's (tile, view) records, which depend on the geometry, the
 * image grid and the view angles only; diff / idiff are not batched
 * (CTGPU_ERR_UNSUPPORTED).  Synchronous.  The buffers named by the problems
 * must stay valid while the batch is used. */
int ctgpu_batch_create(const ctgpu_batch_problem* problems, int n_problems, int flags,
                       ctgpu_batch** out);
/* Filters and backprojects every problem (PostProcessing included) on
 * `stream`; stream-ordered, so check with ctgpu_sync.  The first run sets the
 * launch shape (tuned when CTGPU_BATCH_AUTOTUNE) and, with CTGPU_BATCH_GRAPH,
 * captures later runs' work as one CUDA graph. */
int ctgpu_batch_run(ctgpu_batch* b, void* stream);
/* the launch shape in use: resident blocks per SM and views per pipeline stage cap */
int ctgpu_batch_shape(const ctgpu_batch* b, int* blocks_per_sm, int* views_per_stage);
void ctgpu_batch_destroy(ctgpu_batch* b);

/* Projections::interpolateToParallel (libctsim/projections.cpp:1250-1328),
 * what Reconstructor's bRebinToParallel does (reconstruct.cpp:56): fan-beam
 * d_sino [n_view][pitch] with its view angles -> parallel projections
 * d_out [n_view][out_pitch] over 2 pi (rot_inc 2 pi / n_view), detectors
 * spanning the view diameter; g_out receives their geometry and
 * h_out_angles[n_view] their view angles.  Parallel input is copied. */
int ctgpu_interpolate_to_parallel(const ctgpu_geometry* g, const float* d_sino, int sino_pitch,
                                  const double* h_view_angles, float* d_out, int out_pitch,
                                  ctgpu_geometry* g_out, double* h_out_angles, void* stream);

/* ------------------------------------------------------------------------ */
/* Helical -- replaces Projections::Helical180LI / Helical180LI_Equiangular */
/* and HalfScanFeather (libctsim/projections.cpp:200-439)                     */
/* ------------------------------------------------------------------------ */
/* number of output views, or the reference's error status (1: not enough
 * data, 2: geometry not supported) as CTGPU_ERR_INVALID with a message */
int ctgpu_helical180li_size(const ctgpu_geometry* g, int n_view_in, int interp_view,
                            int* n_view_out);
/* d_in [n_view_in][pitch] -> d_out [n_view_out][pitch]; FP64 weights,
 * reference's FP32 accumulation order; h_out_angles[n_view_out] */
int ctgpu_helical180li(const ctgpu_geometry* g, const float* d_in, int n_view_in, int interp_view,
                       float* d_out, int pitch, double* h_out_angles, int* n_view_out,
                       void* stream);
/* in place on d_data [n_view][pitch] */
int ctgpu_halfscan_feather(const ctgpu_geometry* g, float* d_data, int n_view, int pitch,
                           void* stream);
/* The equilinear restatement of Helical180LI and HalfScanFeather (no
 * reference counterpart: the reference refuses equilinear data,
 * projections.cpp:214-218): the same algorithm with each detector's true fan
 * angle gamma = atan(pos / SDL), pos = (id - (n_det-1)/2) * det_inc; needs
 * equilinear projections.  Arguments as the equiangular entry points. */
int ctgpu_helical180li_equilinear_size(const ctgpu_geometry* g, int n_view_in, int interp_view,
                                       int* n_view_out);
int ctgpu_helical180li_equilinear(const ctgpu_geometry* g, const float* d_in, int n_view_in,
                                  int interp_view, float* d_out, int pitch,
                                  double* h_out_angles, int* n_view_out, void* stream);
int ctgpu_halfscan_feather_equilinear(const ctgpu_geometry* g, float* d_data, int n_view,
                                      int pitch, void* stream);
/* Helical180LI (+ HalfScanFeather) at many interpolation views of one helical
 * data set of n_view_in views.  The FP64 weights and complementary rays of an
 * output sample depend only on the geometry, so the plan tabulates them once;
 * a run then interpolates every slice in one launch, with the same values as
 * ctgpu_helical180li (+ ctgpu_halfscan_feather) slice by slice.  No reference
 * counterpart as one call (pjHinterp does one interpolation view). */
typedef struct ctgpu_helical_plan ctgpu_helical_plan;
#define CTGPU_HELICAL_EQUILINEAR 1   /* the equilinear restatement above */
#define CTGPU_HELICAL_FEATHER 2      /* follow each slice's 180LI by HalfScanFeather */
int ctgpu_helical_plan_create(const ctgpu_geometry* g, int n_view_in, int flags,
                              ctgpu_helical_plan** out);
/* views of every output slice: (pi + fan) / rot_inc + 1 */
int ctgpu_helical_plan_views(const ctgpu_helical_plan* p, int* n_view_out);
/* d_in [n_view_in][in_pitch]; slice z interpolated at view interp_views[z]
 * into d_out + z * out_slice_stride ([n_view_out][out_pitch]); its view angles
 * to h_out_angles[z * n_view_out ..] when non-NULL */
int ctgpu_helical_plan_run(ctgpu_helical_plan* p, const float* d_in, int in_pitch,
                           const int* h_interp_views, int n_slices, float* d_out, int out_pitch,
                           long long out_slice_stride, double* h_out_angles, void* stream);
void ctgpu_helical_plan_destroy(ctgpu_helical_plan* p);

/* ------------------------------------------------------------------------ */
/* Polar and direct-Fourier images -- Projections::convertPolar /            */
/* convertFFTPolar (libctsim/projections.cpp:953-1180) and the GUI's Fourier */
/* reconstruction (src/views.cpp:2828-2849).  Fan-beam data is rebinned to   */
/* parallel rays first (interpolateToParallel), as there; h_view_angles is   */
/* needed for that only.  interp_name: "nearest" | "bilinear" (the           */
/* reference's table; its "bicubic" is commented out).  The reference's      */
/* interpolatePolar loops ix over ny (projections.cpp:1151): columns ix >= ny */
/* are not computed there and are zero here.  Synchronous.                   */
/* ------------------------------------------------------------------------ */
/* convertPolar: d_image [nx][ny] FP32 */
int ctgpu_convert_polar(const ctgpu_geometry* g, const float* d_sino, int pitch,
                        const double* h_view_angles, int nx, int ny, const char* interp_name,
                        float* d_image, void* stream);
/* convertFFTPolar: the complex image as d_real, d_imag [nx][ny] FP32;
 * *n_transform (may be NULL) = the zero-padded transform length
 * (addZeropadFactor of floor(sqrt(nx^2 + ny^2))); FP32 transforms where the
 * reference uses FFTW in FP64 (which this library does not need). */
int ctgpu_convert_fft_polar(const ctgpu_geometry* g, const float* d_sino, int pitch,
                            const double* h_view_angles, int nx, int ny, const char* interp_name,
                            int zeropad, float* d_real, float* d_imag, int* n_transform,
                            void* stream);
/* ImageFile::ifft (backward 2-D DFT after shuffleNaturalToFourierOrder),
 * ImageFile::magnitude and Fourier::shuffleFourierToNaturalOrder of the
 * complex image (d_real, d_imag) into d_out [nx][ny] FP32. */
int ctgpu_image_ifft_magnitude(const float* d_real, const float* d_imag, int nx, int ny,
                               float* d_out, void* stream);
/* the GUI's "Reconstruct Fourier": convertFFTPolar, then ctgpu_image_ifft_magnitude */
int ctgpu_reconstruct_fourier(const ctgpu_geometry* g, const float* d_sino, int pitch,
                              const double* h_view_angles, int nx, int ny,
                              const char* interp_name, int zeropad, float* d_image,
                              void* stream);

/* ------------------------------------------------------------------------ */
/* Files on device-resident data -- .pj / .if I/O (libctsim/projections.cpp: */
/* 485-889, libctsim/array2dfile.cpp:399-640) and the pj2if / if2 utilities  */
/* (tools/pj2if.cpp, tools/if2.cpp, libctsim/imagefile.cpp:186-528).  The    */
/* *_device calls stream the file through page-locked buffers and return     */
/* once the data is in place (they synchronise `stream`).                    */
/* ------------------------------------------------------------------------ */
typedef struct {
  ctgpu_geometry geometry;   /* n_view, n_det, geometry and the scan fields */
  double calc_time;
  int32_t date[6];           /* year, month, day, hour, minute, second */
  int32_t header_size;       /* bytes before the first view record */
  int32_t remark_length;
} ctgpu_pj_info;

/* Projections::read's header part (projections.cpp:553-640): the fields and
 * the remark (NUL-terminated, cut to remark_capacity - 1 bytes; may be NULL). */
int ctgpu_pj_read_header(const char* filename, ctgpu_pj_info* info, char* remark,
                         int remark_capacity);
/* Projections::read's view records (detarrayRead, projections.cpp:811-843)
 * straight into d_sino [n_view][pitch] (pad columns zeroed) and d_angles
 * [n_view].  A file that ends early keeps the whole records it has, like the
 * reference, the rest are zeroed, and *n_views_read (may be NULL) says how
 * many were read.  A record whose detector count differs from the header's
 * fails with CTGPU_ERR_IO (the reference would read past the row). */
int ctgpu_pj_read_device(const char* filename, float* d_sino, int pitch, double* d_angles,
                         int* n_views_read, void* stream);
/* Projections::write (projections.cpp:780-889) from d_sino [n_view][pitch]
 * and d_angles: header from info (header_size and remark_length are derived)
 * and remark; byte-identical to the reference's file for the same values. */
int ctgpu_pj_write_device(const char* filename, const ctgpu_pj_info* info, const char* remark,
                          const float* d_sino, int pitch, const double* d_angles, void* stream);

/* The view records alone, device to device: what detarrayWrite /
 * detarrayRead (projections.cpp:811-889) put in a file after the header,
 * n_view x (12 + 4 n_det) bytes at d_records (4-byte aligned) -- for callers
 * that move the bytes themselves (their own file layer, a socket, a mapped
 * file).  Unpack: d_status [2] must start as {0, 0xffffffff}; it receives the
 * number of records whose detector count differs from n_det and the first
 * such view; pad columns are zeroed. */
int ctgpu_pj_pack(const float* d_sino, int pitch, const double* d_angles, int n_view, int n_det,
                  void* d_records, void* stream);
int ctgpu_pj_unpack(const void* d_records, int n_view, int n_det, float* d_sino, int pitch,
                    double* d_angles, unsigned int* d_status, void* stream);

typedef struct {
  int32_t nx, ny;
  int32_t pixel_format;      /* 7 FP32, 8 FP64 (include/array2dfile.h:118-127) */
  int32_t pixel_size;        /* bytes: 4 or 8 */
  int32_t data_type;         /* 1 real, 2 complex */
  int32_t n_labels;
  int32_t increment_known, extent_known;
  double increment[2];       /* x, y */
  double extent[4];          /* xmin, xmax, ymin, ymax */
  double offset_pv, scale_pv;
  int32_t header_size;
  int32_t reserved;
} ctgpu_if_info;

typedef struct {
  int32_t type;              /* 1 history, 2 user (include/array2dfile.h:49-51) */
  int32_t date[6];           /* all zero on writing: the current local time */
  double calc_time;
  const char* text;
  int32_t text_length;       /* <= 0 on writing: strlen(text) */
  int32_t reserved;
} ctgpu_if_label;

/* Array2dFile::headerRead (array2dfile.cpp:399-439) */
int ctgpu_if_read_header(const char* filename, ctgpu_if_info* info);
/* Array2dFile::labelsRead (array2dfile.cpp:559-595): up to `capacity` labels,
 * their texts NUL-terminated in `text` (label.text NULL where it is full);
 * *n_labels = the labels in the file. */
int ctgpu_if_read_labels(const char* filename, ctgpu_if_label* labels, int capacity, char* text,
                         size_t text_capacity, int* n_labels);
/* Array2dFile::arrayDataRead (array2dfile.cpp:511-549): the real pixels,
 * column-major, into d_image [nx][ny] as FP32 (FP64 files are converted on
 * the device); other pixel formats return CTGPU_ERR_UNSUPPORTED. */
int ctgpu_if_read_device(const char* filename, float* d_image, void* stream);
/* Array2dFile::fileWrite (array2dfile.cpp:443-509, :598-640) of the FP32 real
 * image d_image [nx][ny] with info's axes and the labels given. */
int ctgpu_if_write_device(const char* filename, const ctgpu_if_info* info,
                          const ctgpu_if_label* labels, int n_labels, const float* d_image,
                          void* stream);
/* pj2if (tools/pj2if.cpp:118-125): d_image [n_det][n_view] column-major with
 * v[ix][iy] = row n_view - 1 - iy, detector ix of d_sino [n_view][pitch]. */
int ctgpu_sino_to_image(const float* d_sino, int pitch, int n_view, int n_det, float* d_image,
                        void* stream);
/* ImageFile::comparativeStatistics (imagefile.cpp:186-240), what if2 --comp
 * prints, for n_images pairs (d_a + i * image_stride, d_b + i * image_stride)
 * of nx x ny images: h_dre[3 i ..] = d, r, e.  e is exact; d and r agree with
 * the reference's sequential FP64 sums to about 1e-12 relative and do not
 * depend on timing.  An image smaller than 2 x 2 gives e = -1 as there. */
int ctgpu_image_compare(const float* d_a, const float* d_b, int n_images, int nx, int ny,
                        size_t image_stride, double* h_dre, void* stream);
/* The same with the results left in device memory (d_dre [n_images][3]):
 * enqueued on `stream`, no synchronisation (its few KB of scratch are
 * allocated and freed stream-ordered).  nx * ny must be below 2^31. */
int ctgpu_image_compare_device(const float* d_a, const float* d_b, int n_images, int nx, int ny,
                               size_t image_stride, double* d_dre, void* stream);
/* ImageFile::addImages / subtractImages / multiplyImages / divideImages
 * (imagefile.cpp:378-528) on real FP32 images: op "add" | "subtract" |
 * "multiply" | "divide"; d_out[i] = d_a[i] op d_b[i] for n pixels.  Division
 * by zero gives inf / nan, as the reference (its zero test is on a pointer). */
int ctgpu_image_arith(const char* op, const float* d_a, const float* d_b, float* d_out, size_t n,
                      void* stream);

/* ------------------------------------------------------------------------ */
/* Allocation-free variant                                                   */
/* ------------------------------------------------------------------------ */
/* No counterpart in the reference.  The "diff" backprojection of
 * ctgpu_recon_backproject for callers that cannot allocate device memory --
 * plug-ins whose host application owns every device allocation (its own
 * allocator or a fixed memory budget), real-time loops that must not block on
 * the allocator.  It calls no cudaMalloc,
 * cudaFree or other allocating routine: the per-view steps and per-(view,
 * column) row ranges the diff backprojector needs live in a fixed 16 MiB
 * device array inside the library, which every GPU that loads the library
 * keeps until the process exits.  The caller passes the filtered sinogram
 * (d_filtered [n_views][filtered_pitch]) and the image (d_image [nx][ny]);
 * g describes a parallel-beam scan, roi may be NULL; flags: CTGPU_RUN_POSTPROCESS
 * applies PostProcessing's rotScale, CTGPU_RUN_ACCUMULATE adds to d_image.
 * Limits: 24*n_views + 16*n_views*nx bytes (+ alignment) must fit in 16 MiB,
 * about a million view-columns (e.g. 1440 views x 704 columns); larger
 * requests return CTGPU_ERR_INVALID with the size needed.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture.  All calls
 * share the array and it keeps the last call's contents (each call rewrites
 * everything it reads); calls that overlap on the GPU, on different streams
 * or threads, race on it.  The view angles are read on the host during the
 * call; the per-view steps reach the array as kernel parameters, so no host
 * buffer is read after the call returns. */
int ctgpu_backproject_diff_noalloc(const ctgpu_geometry* g, int nx, int ny,
                                   const char* interp_name, const ctgpu_roi* roi,
                                   const float* d_filtered, int filtered_pitch,
                                   const double* h_view_angles, int n_views, float* d_image,
                                   int flags, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CTGPU_H */
