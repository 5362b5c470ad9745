/* ctoracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 CPU restatement of CTSim's simulate-and-reconstruct path, used as the
 * checker for the GPU library (tests/, __graft_entry__.smoke(), bench.py's CPU
 * baseline).  The product never links, loads or calls this code.
 *
 * Every function cites the CTSim file:line it restates.  Images are FP64 (the
 * reference compiled with IMAGEFILE_64_BITS); sinograms are produced in FP64
 * and the reference's FP32 storage is applied by the caller where needed.
 *
 * Parity of this restatement against the reference itself is pinned by the
 * golden fixtures in tests/golden/ (made by tests/golden/make_golden.py from
 * the reference compiled from source by oracle/Makefile).
 */
#ifndef CTORACLE_H
#define CTORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* element types: include/phantom.h:34-41 */
enum { ORA_PELEM_INVALID = 0, ORA_PELEM_RECTANGLE, ORA_PELEM_TRIANGLE, ORA_PELEM_ELLIPSE,
       ORA_PELEM_SECTOR, ORA_PELEM_SEGMENT };
/* geometries: libctsim/scanner.cpp:29-33 */
enum { ORA_GEOM_PARALLEL = 0, ORA_GEOM_EQUIANGULAR = 1, ORA_GEOM_EQUILINEAR = 2 };
/* backprojectors / interpolation: libctsim/backprojectors.cpp:28-60 */
enum { ORA_BP_TRIG = 0, ORA_BP_TABLE, ORA_BP_DIFF, ORA_BP_IDIFF };
enum { ORA_INTERP_NEAREST = 0, ORA_INTERP_LINEAR, ORA_INTERP_CUBIC };
/* filter methods: libctsim/procsignal.cpp:33-41 ("fft" here = FFTW's math) */
enum { ORA_FM_CONVOLUTION = 0, ORA_FM_FOURIER, ORA_FM_FOURIER_TABLE, ORA_FM_FFT };
enum { ORA_FG_DIRECT = 0, ORA_FG_INVERSE_FOURIER };

typedef struct {
  int type;
  double cx, cy, u, v, rot, atten;      /* rot in radians */
  double xmin, xmax, ymin, ymax;        /* outline-polygon bounding box */
  double phm2obj[3][3], obj2phm[3][3];  /* row-vector affine maps */
} ora_pelem;

typedef struct {
  int n;               /* number of elements */
  int unit_pulse;      /* composition P_UNIT_PULSE */
  int cap;             /* elements e has room for (grown by ora_phantom_add) */
  ora_pelem* e;        /* in the reference's list order (last added first) */
  double xmin, xmax, ymin, ymax;
} ora_phantom;

typedef struct {
  int fail;
  int geometry, nDet, nView, offsetView, nSample;
  double rotLen, rotInc, detInc, detLen, detStart;
  double viewDiameter, scanDiameter, focalLength, centerDetectorLength, sourceDetectorLength;
  double fanBeamAngle, xCenter, yCenter, angularDetLen, angularDetInc;
  double xs1, ys1, xs2, ys2, xd1, yd1, xd2, yd2;
  double incmtx[3][3];
} ora_scanner;

typedef struct {
  int fail;
  int filterId, method, generation, geometry;
  int nSignal, nFilterPoints, nOutput, zeropad, interpFactor;
  double signalInc, bandwidth, param, focalLength, sdl;
  double* filter;      /* nFilterPoints */
  double *cosTable, *sinTable; int nTable;
} ora_procsig;

typedef struct {
  int geometry, nDet, nView;
  double rotInc, detInc, focalLength, sourceDetectorLength, viewDiameter, fanBeamAngle;
} ora_geom;

/* ---- phantom ---- */
int  ora_name_to_pelem_type(const char* name);
int  ora_phantom_init(ora_phantom* p, int maxElems);
int  ora_phantom_add(ora_phantom* p, int type, double cx, double cy, double u, double v,
                     double rotDeg, double atten);
int  ora_phantom_builtin(ora_phantom* p, const char* name);
void ora_phantom_free(ora_phantom* p);

/* ---- scanner / ray-sums ---- */
int  ora_geometry_id(const char* name);
int  ora_scanner_init(ora_scanner* s, const ora_phantom* p, int geometry, int nDet, int nView,
                      int offsetView, int nSample, double rotAngle, double flRatio, double cdRatio,
                      double viewRatio, double scanRatio);
void ora_collect_projections(const ora_scanner* s, const ora_phantom* p, int iStartView,
                             int iNumViews, int iOffsetView, int iStorageOffset, double* sino,
                             double* viewAngles, int nThreads);
double ora_raysum(const ora_phantom* p, double x1, double y1, double x2, double y2);
/* d(sum gsino * sino)/d(cx, cy, u, v, rot radians, atten) of the ellipses
 * (list order), FP64; gsino [nView][nDet]; grad [6 * n] */
void ora_ellipse_gradient(const ora_scanner* s, const ora_phantom* p, const double* gsino,
                          double* grad);
/* helical scan of a 3-D ellipsoid phantom (restatement only); ell[8k..8k+7] =
 * cx, cy, cz, a, b, c, rot_deg, atten; view v sees z = z0 + v dz */
void ora_collect_ellipsoids(const ora_scanner* s, const double* ell, int n, double z0, double dz,
                            double* sino, double* viewAngles, int nThreads);

/* ---- filtering ---- */
int  ora_filter_id(const char* name);
int  ora_filter_method_id(const char* name);
int  ora_filter_generation_id(const char* name);
int  ora_procsig_init(ora_procsig* ps, int filterId, int method, double bandwidth, double signalInc,
                      int nSignal, double param, int generation, int zeropad, int interpFactor,
                      int geometry, double focalLength, double sdl);
void ora_procsig_free(ora_procsig* ps);
void ora_filter_signal(const ora_procsig* ps, const float* in, double* out);
void ora_filter_views(const ora_procsig* ps, const float* sino, int nView, double* out,
                      int nThreads);
double ora_frequency_response(int filterId, double bw, double u, double param);
double ora_spatial_response(int filterId, double bw, double x, double param);

/* ---- backprojection ---- */
int  ora_backproject(const ora_geom* g, const double* filtered, int filtStride,
                     const double* viewAngles, int iStartView, int nViewsBP, int nx, int ny,
                     const double* roi, int bproj, int interp, double* image, int postProcess,
                     int nThreads);
double ora_cubic_interpolate(const double* y, int n, double x);

/* ---- reconstruction (filter + backproject), reference defaults ---- */
int  ora_reconstruct(const ora_geom* g, const float* sino, const double* viewAngles, int nx,
                     int ny, int filterId, double param, int method, int zeropad, int generation,
                     int bproj, int interp, double* image, int nThreads);

/* ---- helical ---- */
int  ora_helical180li(const ora_geom* g, const float* in, int nViewIn, int interpView,
                      float* out, double* outAngles, int* nViewOut);
int  ora_halfscan_feather(const ora_geom* g, float* data, int nView);
/* the same, with the equilinear restatement allowed / the true equilinear fan angle */
int  ora_helical180li_ex(const ora_geom* g, const float* in, int nViewIn, int interpView,
                         float* out, double* outAngles, int* nViewOut, int allowEquilinear);
int  ora_halfscan_feather_ex(const ora_geom* g, float* data, int nView, int trueGamma);

/* ---- rebinning to parallel rays: Projections::interpolateToParallel ---- */
/* fan-beam in [nView][nDet] with its view angles, rotStart and detStart (the
 * .pj header's) -> out [nView][nDet], outAngles[nView], outHdr = {rotInc,
 * detStart, detInc} of the parallel projections; 1 for parallel input */
int ora_interpolate_to_parallel(const ora_geom* g, double rotStart, double detStart,
                                const float* in, const double* viewAngles, float* out,
                                double* outAngles, double* outHdr);

/* ---- rasteriser (phm2if) and pixel-image projector ---- */
void ora_phantom_to_image(const ora_phantom* p, int nx, int ny, double viewRatio, int nsample,
                          double* image, double extent[4], int nThreads);
int  ora_project_image(const ora_geom* g, const double* image, int nx, int ny,
                       const double* viewAngles, int nView, double* sino, int nThreads);

/* ---- polar / direct-Fourier images (Projections::convertPolar /
   convertFFTPolar, the GUI's Fourier reconstruction) ---- */
/* interp: 0 nearest, 1 bilinear; out [nx][ny]; fan-beam input is rebinned
   first (interpolateToParallel) */
int  ora_convert_polar(const ora_geom* g, double rotStart, double detStart, const float* sino,
                       const double* angles, int nx, int ny, int interp, float* out);
int  ora_add_zeropad_factor(int n, int zeropad);
/* returns the zero-padded transform length */
int  ora_convert_fft_polar(const ora_geom* g, double rotStart, double detStart,
                           const float* sino, const double* angles, int nx, int ny, int interp,
                           int zeropad, float* outRe, float* outIm);
/* ImageFile::ifft, magnitude, Fourier::shuffleFourierToNaturalOrder */
void ora_ifft_magnitude(const float* inRe, const float* inIm, int nx, int ny, float* out);

/* ---- if2 --comp: ImageFile::comparativeStatistics -> out = {d, r, e}; 0 if empty ---- */
int ora_image_compare(const float* a, const float* b, int nx, int ny, double out[3]);

#ifdef __cplusplus
}
#endif
#endif
