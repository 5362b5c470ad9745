// Test infrastructure only: a small driver linked against the unmodified CTSim
// library objects (built by `make ref` into oracle/_ref/).  It exposes, as raw
// binary dumps, the intermediate results the CLIs do not write out, so the
// FP64 restatement in ctoracle.c and the GPU path can be pinned to the
// reference's own numbers:
//
//   ref_harness filter  GEOM NDET NVIEW DETINC FL SDL FILTER PARAM METHOD ZEROPAD GEN INTERPF in.f32 out.f64
//       ProcessSignal::filterSignal on every row  (libctsim/procsignal.cpp:543)
//   ref_harness bp      PJFILE filtered.f64 NX NY BACKPROJ INTERP out.f64 [XMIN YMIN XMAX YMAX]
//       Backprojector::BackprojectView per view + PostProcessing
//       (libctsim/backprojectors.cpp:109-121), optionally with a
//       ReconstructionROI (:284-315)
//   ref_harness timerec PJFILE NX NY FILTER METHOD BACKPROJ INTERP NTHREADS [NVIEWS [PARAM [ZEROPAD]]]
//       times Reconstructor over the first NVIEWS views, split across NTHREADS
//       threads the way the GUI's worker threads do (one Reconstructor and one
//       private image per thread, images summed: src/threadrecon.cpp:176-255)
//   ref_harness rebin   IN.pj OUT.pj
//       Projections::interpolateToParallel (libctsim/projections.cpp:1250-1328)
//   ref_harness polar   PJFILE NX NY INTERP out.f32
//       Projections::convertPolar (libctsim/projections.cpp:953-995) into a
//       cleared FP32 ImageFile, dumped column-major
//   ref_harness comp    A.if B.if
//       ImageFile::comparativeStatistics (libctsim/imagefile.cpp:186-240),
//       printed as "d r e" with 17 significant digits
//   ref_harness timeraysum PHM NDET NVIEW NRAY GEOM NTHREADS [NVIEWS]
//       times Scanner::collectProjections over view sub-ranges per thread
//       (libctsim/scanner.cpp:295-298)
#include "ct.h"
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <omp.h>

static bool readRaw(const char* fn, void* p, size_t n) {
  FILE* f = fopen(fn, "rb");
  if (!f) return false;
  size_t r = fread(p, 1, n, f);
  fclose(f);
  return r == n;
}
static bool writeRaw(const char* fn, const void* p, size_t n) {
  FILE* f = fopen(fn, "wb");
  if (!f) return false;
  size_t w = fwrite(p, 1, n, f);
  fclose(f);
  return w == n;
}

static int cmdFilter(int argc, char** argv) {
  if (argc != 16) { fprintf(stderr, "filter: bad args\n"); return 2; }
  int geom = atoi(argv[2]), nDet = atoi(argv[3]), nView = atoi(argv[4]);
  double detInc = atof(argv[5]), fl = atof(argv[6]), sdl = atof(argv[7]);
  const char* filt = argv[8];
  double param = atof(argv[9]);
  const char* method = argv[10];
  int zeropad = atoi(argv[11]);
  const char* gen = argv[12];
  int interpF = atoi(argv[13]);
  std::vector<float> in((size_t)nView * nDet);
  if (!readRaw(argv[14], in.data(), in.size() * 4)) { fprintf(stderr, "read fail\n"); return 2; }
  ProcessSignal ps(filt, method, 1. / detInc, detInc, nDet, param, "spatial", gen, zeropad, interpF, 0,
                   geom, fl, sdl);
  if (ps.fail()) { fprintf(stderr, "ProcessSignal: %s\n", ps.failMessage().c_str()); return 3; }
  size_t nOut = (size_t)nDet * interpF;
  std::vector<double> out((size_t)nView * nOut);
  for (int v = 0; v < nView; v++) ps.filterSignal(&in[(size_t)v * nDet], &out[(size_t)v * nOut]);
  return writeRaw(argv[15], out.data(), out.size() * 8) ? 0 : 2;
}

static int cmdBackproject(int argc, char** argv) {
  if (argc != 9 && argc != 13) { fprintf(stderr, "bp: bad args\n"); return 2; }
  ReconstructionROI roi;
  const bool haveRoi = argc == 13;
  if (haveRoi) {
    roi.m_dXMin = atof(argv[9]);
    roi.m_dYMin = atof(argv[10]);
    roi.m_dXMax = atof(argv[11]);
    roi.m_dYMax = atof(argv[12]);
  }
  Projections pj;
  if (!pj.read(argv[2])) { fprintf(stderr, "pj read fail\n"); return 2; }
  int nx = atoi(argv[4]), ny = atoi(argv[5]);
  int nDet = pj.nDet(), nView = pj.nView();
  std::vector<double> filt((size_t)nView * nDet);
  if (!readRaw(argv[3], filt.data(), filt.size() * 8)) { fprintf(stderr, "read fail\n"); return 2; }
  ImageFile im(nx, ny);
  Backprojector bp(pj, im, argv[6], argv[7], 1, haveRoi ? &roi : NULL);
  if (bp.fail()) { fprintf(stderr, "Backprojector: %s\n", bp.failMessage().c_str()); return 3; }
  for (int v = 0; v < nView; v++)
    bp.BackprojectView(&filt[(size_t)v * nDet], pj.getDetectorArray(v).viewAngle());
  bp.PostProcessing();
  std::vector<double> out((size_t)nx * ny);
  ImageFileArray a = im.getArray();
  for (int ix = 0; ix < nx; ix++)
    for (int iy = 0; iy < ny; iy++) out[(size_t)ix * ny + iy] = a[ix][iy];
  return writeRaw(argv[8], out.data(), out.size() * 8) ? 0 : 2;
}

static int cmdTimeRec(int argc, char** argv) {
  if (argc < 10) { fprintf(stderr, "timerec: bad args\n"); return 2; }
  Projections pj;
  if (!pj.read(argv[2])) { fprintf(stderr, "pj read fail\n"); return 2; }
  int nx = atoi(argv[3]), ny = atoi(argv[4]);
  const char *filt = argv[5], *method = argv[6], *bproj = argv[7], *interp = argv[8];
  int nThreads = atoi(argv[9]);
  int nViews = argc > 10 ? atoi(argv[10]) : pj.nView();
  if (nViews > pj.nView()) nViews = pj.nView();
  double param = argc > 11 ? atof(argv[11]) : -1;
  int zeropad = argc > 12 ? atoi(argv[12]) : 1;
  std::vector<ImageFile*> ims(nThreads);
  auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel num_threads(nThreads)
  {
    int t = omp_get_thread_num();
    int per = nViews / nThreads, extra = nViews % nThreads;
    int start = t * per + (t < extra ? t : extra);
    int count = per + (t < extra ? 1 : 0);
    ims[t] = new ImageFile(nx, ny);
    Reconstructor rec(pj, *ims[t], filt, param, method, zeropad, "direct", interp, 1, bproj, 0);
    if (count > 0) rec.reconstructView(start, count);
    rec.postProcessing();
  }
  ImageFileArray sum = ims[0]->getArray();
  for (int t = 1; t < nThreads; t++) {
    ImageFileArray a = ims[t]->getArray();
    for (int ix = 0; ix < nx; ix++)
      for (int iy = 0; iy < ny; iy++) sum[ix][iy] += a[ix][iy];
  }
  double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  printf("{\"seconds\": %.6f, \"pixel_view_updates\": %.0f, \"pv_per_s\": %.6e, \"threads\": %d, \"views\": %d}\n",
         s, (double)nx * ny * nViews, (double)nx * ny * nViews / s, nThreads, nViews);
  for (int t = 0; t < nThreads; t++) delete ims[t];
  return 0;
}

static int cmdTimeRaysum(int argc, char** argv) {
  if (argc < 8) { fprintf(stderr, "timeraysum: bad args\n"); return 2; }
  Phantom phm;
  if (!phm.createFromPhantom(argv[2])) phm.createFromFile(argv[2]);
  int nDet = atoi(argv[3]), nView = atoi(argv[4]), nRay = atoi(argv[5]);
  const char* geom = argv[6];
  int nThreads = atoi(argv[7]);
  int nViews = argc > 8 ? atoi(argv[8]) : nView;
  double rot = (strcmp(geom, "parallel") == 0 ? 0.5 : 1.0) * TWOPI;
  Scanner sc(phm, geom, nDet, nView, 0, nRay, rot, 2., 2., 1., 1.);
  if (sc.fail()) { fprintf(stderr, "Scanner: %s\n", sc.failMessage().c_str()); return 3; }
  Projections pj(sc);
  auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel num_threads(nThreads)
  {
    int t = omp_get_thread_num();
    int per = nViews / nThreads, extra = nViews % nThreads;
    int start = t * per + (t < extra ? t : extra);
    int count = per + (t < extra ? 1 : 0);
    Scanner mine(phm, geom, nDet, nView, 0, nRay, rot, 2., 2., 1., 1.);
    if (count > 0) mine.collectProjections(pj, phm, start, count, 0, true, 0);
  }
  double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  printf("{\"seconds\": %.6f, \"raysums\": %.0f, \"raysums_per_s\": %.6e, \"threads\": %d, \"views\": %d}\n",
         s, (double)nDet * nViews, (double)nDet * nViews / s, nThreads, nViews);
  return 0;
}

static int cmdRebin(int argc, char** argv) {
  if (argc != 4) { fprintf(stderr, "rebin: bad args\n"); return 2; }
  Projections p;
  if (!p.read(argv[2])) { fprintf(stderr, "read fail\n"); return 2; }
  Projections* q = p.interpolateToParallel();
  bool ok = q->write(argv[3]);
  if (q != &p) delete q;
  return ok ? 0 : 2;
}

static int cmdPolar(int argc, char** argv) {
  if (argc < 7) return 2;
  Projections pj;
  if (!pj.read(argv[2])) { fprintf(stderr, "pj read fail\n"); return 2; }
  int nx = atoi(argv[3]), ny = atoi(argv[4]);
  ImageFile im(nx, ny);
  im.arrayDataClear();
  if (!pj.convertPolar(im, Projections::convertInterpNameToID(argv[5]))) return 3;
  std::vector<float> out((size_t)nx * ny);
  ImageFileArray v = im.getArray();
  for (int ix = 0; ix < nx; ix++)
    for (int iy = 0; iy < ny; iy++) out[(size_t)ix * ny + iy] = v[ix][iy];
  return writeRaw(argv[6], out.data(), out.size() * 4) ? 0 : 2;
}

static int cmdComp(int argc, char** argv) {
  if (argc < 4) return 2;
  ImageFile a, b;
  if (!a.fileRead(argv[2]) || !b.fileRead(argv[3])) { fprintf(stderr, "if read fail\n"); return 2; }
  double d = 0, r = 0, e = 0;
  if (!a.comparativeStatistics(b, d, r, e)) { printf("false\n"); return 0; }
  printf("%.17g %.17g %.17g\n", d, r, e);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) { fprintf(stderr, "usage: ref_harness filter|bp|timerec|timeraysum|rebin|comp|polar ...\n"); return 2; }
  std::string c = argv[1];
  if (c == "filter") return cmdFilter(argc, argv);
  if (c == "bp") return cmdBackproject(argc, argv);
  if (c == "timerec") return cmdTimeRec(argc, argv);
  if (c == "timeraysum") return cmdTimeRaysum(argc, argv);
  if (c == "rebin") return cmdRebin(argc, argv);
  if (c == "comp") return cmdComp(argc, argv);
  if (c == "polar") return cmdPolar(argc, argv);
  fprintf(stderr, "unknown command %s\n", argv[1]);
  return 2;
}
