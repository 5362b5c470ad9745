// ctsim_api.cpp -- the drop-in C++ classes of include/ctsim_gpu.h, implemented on
// the C ABI (include/ctgpu.h).  File formats: .pj (libctsim/projections.cpp:
// 485-637, :816-889) and .if (libctsim/array2dfile.cpp:400-600), little-endian.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>
#include <strings.h>

#include <cuda_runtime.h>

#include "../../include/ctsim_gpu.h"

static_assert(sizeof(double) == 8 && sizeof(float) == 4, "IEEE sizes expected");

namespace {

std::string last_err() { return std::string(ctgpu_last_error()); }

// little-endian stream helpers (this library targets little-endian hosts)
template <class T>
void put(std::string& b, T v) {
  b.append(reinterpret_cast<const char*>(&v), sizeof(T));
}
template <class T>
bool get(const std::vector<char>& b, size_t& off, T& v) {
  if (off + sizeof(T) > b.size()) return false;
  std::memcpy(&v, b.data() + off, sizeof(T));
  off += sizeof(T);
  return true;
}
bool slurp(const char* fn, std::vector<char>& b) {
  std::ifstream f(fn, std::ios::binary);
  if (!f) return false;
  b.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  return true;
}
void now_date(int d[6]) {   // Array2dFileLabel::init / Projections::init (struct tm fields)
  time_t t = time(nullptr);
  tm* lt = localtime(&t);
  d[0] = lt->tm_year; d[1] = lt->tm_mon; d[2] = lt->tm_mday;
  d[3] = lt->tm_hour; d[4] = lt->tm_min; d[5] = lt->tm_sec;
}

}  // namespace

// ================================================================ Phantom ==
Phantom::Phantom() : m_h(nullptr), m_fail(false) { ctgpu_phantom_create(&m_h); }
Phantom::Phantom(const char* phmName) : m_h(nullptr), m_fail(false) {
  ctgpu_phantom_create(&m_h);
  createFromPhantom(phmName);
}
Phantom::~Phantom() { ctgpu_phantom_destroy(m_h); }

bool Phantom::createFromPhantom(const char* phmName) {
  ctgpu_phantom* p = nullptr;
  if (ctgpu_phantom_create_builtin(phmName, &p) != CTGPU_OK) {
    m_fail = true;
    m_failMessage = last_err();
    return false;
  }
  ctgpu_phantom_destroy(m_h);
  m_h = p;
  m_name = phmName;
  return true;
}

bool Phantom::createFromFile(const char* fname) {
  if (ctgpu_phantom_read_file(m_h, fname) != CTGPU_OK) {
    m_failMessage = last_err();
    return false;
  }
  m_name = fname;
  return true;
}

void Phantom::addPElem(const char* type, double cx, double cy, double u, double v, double rot,
                       double atten) {
  if (ctgpu_phantom_add_element(m_h, type, cx, cy, u, v, rot, atten) != CTGPU_OK)
    std::fprintf(stderr, "Warning: %s [Phantom::addPElem]\n", ctgpu_last_error());
}

static double bound(ctgpu_phantom* h, int k) {
  double b[4] = {0, 0, 0, 0};
  ctgpu_phantom_bounds(h, b, nullptr);
  return b[k];
}
int Phantom::nPElem() const {
  int n = 0;
  ctgpu_phantom_bounds(m_h, nullptr, &n);
  return n;
}
double Phantom::xmin() const { return bound(m_h, 0); }
double Phantom::xmax() const { return bound(m_h, 1); }
double Phantom::ymin() const { return bound(m_h, 2); }
double Phantom::ymax() const { return bound(m_h, 3); }
double Phantom::maxAxisLength() const {
  double dx = xmax() - xmin(), dy = ymax() - ymin();
  return dx > dy ? dx : dy;
}
double Phantom::getDiameterBoundaryCircle() const { return 1.414213562373095049 * maxAxisLength(); }

// ================================================================ Scanner ==
Scanner::Scanner(const Phantom& phm, const char* geometryName, int nDet, int nView,
                 int iOffsetView, int nSample, double rot_anglen, double fl, double cd,
                 double vr, double sr)
    : m_h(nullptr), m_offsetView(iOffsetView), m_fail(false) {
  std::memset(&m_g, 0, sizeof(m_g));
  if (ctgpu_scanner_create(phm.handle(), geometryName, nDet, nView, iOffsetView,
                           nSample < 1 ? 1 : nSample, rot_anglen, fl, cd, vr, sr,
                           &m_h) != CTGPU_OK) {
    m_fail = true;
    m_failMessage = last_err();
    return;
  }
  ctgpu_scanner_geometry(m_h, &m_g);
}
Scanner::~Scanner() { ctgpu_scanner_destroy(m_h); }

int Scanner::convertGeometryNameToID(const char* n) {
  if (!strcasecmp(n, "parallel")) return GEOMETRY_PARALLEL;
  if (!strcasecmp(n, "equiangular")) return GEOMETRY_EQUIANGULAR;
  if (!strcasecmp(n, "equilinear")) return GEOMETRY_EQUILINEAR;
  if (!strcasecmp(n, "linogram")) return 3;
  return GEOMETRY_INVALID;
}
const char* Scanner::convertGeometryIDToName(int id) {
  static const char* names[] = {"parallel", "equiangular", "equilinear", "linogram"};
  return (id >= 0 && id < 4) ? names[id] : "";
}

void Scanner::collectProjections(Projections& proj, const Phantom& phm, int trace, SGP*) {
  collectProjections(proj, phm, 0, proj.nView(), m_offsetView, true, trace);
}
void Scanner::collectProjections(Projections& proj, const Phantom& phm, int iStartView,
                                 int iNumViews, int iOffsetView, bool bStore, int trace, SGP*) {
  collectProjections(proj, phm, iStartView, iNumViews, iOffsetView, bStore ? iStartView : 0, trace);
}
void Scanner::collectProjections(Projections& proj, const Phantom& phm, int iStartView,
                                 int iNumViews, int iOffsetView, int iStorageOffset, int, SGP*) {
  if (m_fail || iNumViews <= 0) return;
  std::vector<float> tmp((size_t)proj.nView() * proj.nDet());
  std::vector<double> ang(proj.nView());
  int rc = ctgpu_collect_projections_host(m_h, phm.handle(), iStartView, iNumViews, iOffsetView,
                                          iStorageOffset, tmp.data(), ang.data());
  if (rc != CTGPU_OK) {
    std::fprintf(stderr, "collectProjections: %s\n", ctgpu_last_error());
    return;
  }
  for (int v = iStorageOffset; v < iStorageOffset + iNumViews && v < proj.nView(); v++) {
    DetectorArray& d = proj.getDetectorArray(v);
    std::memcpy(d.detValues(), &tmp[(size_t)v * proj.nDet()], sizeof(float) * proj.nDet());
    d.setViewAngle(ang[v]);
  }
}

// ============================================================ Projections ==
Projections::Projections() : m_pitch(0), m_calcTime(0) {
  std::memset(&m_g, 0, sizeof(m_g));
  init(0, 0);
}
Projections::Projections(const Scanner& s) : m_pitch(0), m_calcTime(0) { initFromScanner(s); }
Projections::Projections(int nView, int nDet) : m_pitch(0), m_calcTime(0) {
  std::memset(&m_g, 0, sizeof(m_g));
  init(nView, nDet);
}
Projections::~Projections() {}

void Projections::stampDate() { now_date(m_date); }

void Projections::init(int nView, int nDet) {
  m_g.n_view = nView;
  m_g.n_det = nDet;
  m_pitch = (nDet + 3) & ~3;
  m_data.assign((size_t)nView * m_pitch, 0.f);
  m_views.assign(nView, DetectorArray());
  for (int v = 0; v < nView; v++) {
    m_views[v].m_detValues = m_data.data() + (size_t)v * m_pitch;
    m_views[v].m_nDet = nDet;
  }
  stampDate();
}

void Projections::initFromScanner(const Scanner& s) {   // projections.cpp:145-161
  m_g = s.gpuGeometry();
  init(m_g.n_view, m_g.n_det);
}

void Projections::setNView(int nView) { init(nView, m_g.n_det); }

std::vector<double> Projections::viewAngles() const {
  std::vector<double> a(m_g.n_view);
  for (int v = 0; v < m_g.n_view; v++) a[v] = m_views[v].viewAngle();
  return a;
}

bool Projections::read(const char* fn) {   // projections.cpp:553-672
  std::vector<char> b;
  if (!slurp(fn, b)) return false;
  size_t off = 0;
  uint16_t hsize, sig, date[6], rlen;
  uint32_t nView, nDet, geom;
  double d[9];
  if (!get(b, off, hsize) || !get(b, off, sig) || !get(b, off, nView) || !get(b, off, nDet) ||
      !get(b, off, geom))
    return false;
  for (double& x : d)
    if (!get(b, off, x)) return false;
  for (uint16_t& x : date)
    if (!get(b, off, x)) return false;
  if (!get(b, off, rlen)) return false;
  if (sig != 'P' * 256 + 'J' || off + rlen != hsize || hsize > b.size()) return false;
  m_remark.assign(b.data() + off, rlen);
  m_filename = fn;
  m_calcTime = d[0];
  std::memset(&m_g, 0, sizeof(m_g));
  init((int)nView, (int)nDet);
  m_g.geometry = (int)geom;
  m_g.rot_start = d[1]; m_g.rot_inc = d[2]; m_g.det_start = d[3]; m_g.det_inc = d[4];
  m_g.view_diameter = d[5]; m_g.focal_length = d[6]; m_g.source_detector_length = d[7];
  m_g.fan_beam_angle = d[8];
  for (int i = 0; i < 6; i++) m_date[i] = date[i];
  off = hsize;
  for (uint32_t v = 0; v < nView; v++) {
    double a;
    uint32_t nd;
    if (!get(b, off, a) || !get(b, off, nd)) break;
    if (off + 4 * (size_t)nDet > b.size()) break;
    m_views[v].setViewAngle(a);
    std::memcpy(m_views[v].detValues(), b.data() + off, 4 * (size_t)nDet);
    off += 4 * (size_t)nDet;
  }
  return true;
}

bool Projections::write(const char* fn) {   // projections.cpp:485-546, :780-889
  std::string b;
  put<uint16_t>(b, 0);
  put<uint16_t>(b, 'P' * 256 + 'J');
  put<uint32_t>(b, m_g.n_view);
  put<uint32_t>(b, m_g.n_det);
  put<uint32_t>(b, m_g.geometry);
  for (double x : {m_calcTime, m_g.rot_start, m_g.rot_inc, m_g.det_start, m_g.det_inc,
                   m_g.view_diameter, m_g.focal_length, m_g.source_detector_length,
                   m_g.fan_beam_angle})
    put<double>(b, x);
  for (int i = 0; i < 6; i++) put<uint16_t>(b, (uint16_t)m_date[i]);
  put<uint16_t>(b, (uint16_t)m_remark.size());
  b += m_remark;
  uint16_t hs = (uint16_t)b.size();
  std::memcpy(&b[0], &hs, 2);
  for (int v = 0; v < m_g.n_view; v++) {
    put<double>(b, m_views[v].viewAngle());
    put<uint32_t>(b, m_g.n_det);
    b.append(reinterpret_cast<const char*>(m_views[v].detValues()), 4 * (size_t)m_g.n_det);
  }
  std::ofstream f(fn, std::ios::binary | std::ios::trunc);
  if (!f) return false;
  f.write(b.data(), b.size());
  return (bool)f;
}

void Projections::printScanInfo(std::string& out) const {
  std::ostringstream os;   // projections.cpp:935-949
  os << "Number of detectors: " << m_g.n_det << "\n";
  os << "Number of views: " << m_g.n_view << "\n";
  os << "Description: " << m_remark.c_str() << "\n";
  os << "Geometry: " << Scanner::convertGeometryIDToName(m_g.geometry) << "\n";
  os << "Focal Length: " << m_g.focal_length << "\n";
  os << "Source Detector Length: " << m_g.source_detector_length << "\n";
  os << "View Diameter: " << m_g.view_diameter << "\n";
  os << "Fan Beam Angle: " << m_g.fan_beam_angle * (180. / 3.14159265358979323846) << "\n";
  os << "detStart: " << m_g.det_start << "\n";
  os << "detInc: " << m_g.det_inc << "\n";
  os << "rotStart: " << m_g.rot_start << "\n";
  os << "rotInc: " << m_g.rot_inc << "\n";
  out = os.str();
}

void Projections::printProjectionData(int startView, int endView) const {
  std::printf("Projections Data\n\n");   // projections.cpp:905-932
  std::printf("Description: %s\n", m_remark.c_str());
  std::printf("Geometry: %s\n", Scanner::convertGeometryIDToName(m_g.geometry));
  std::printf("nView       = %8d             nDet = %8d\n", m_g.n_view, m_g.n_det);
  std::printf("focalLength = %8.4f   ViewDiameter = %8.4f\n", m_g.focal_length, m_g.view_diameter);
  std::printf("fanBeamAngle= %8.4f SourceDetector = %8.4f\n",
              m_g.fan_beam_angle * (180. / 3.14159265358979323846), m_g.source_detector_length);
  std::printf("rotStart    = %8.4f         rotInc = %8.4f\n", m_g.rot_start, m_g.rot_inc);
  std::printf("detStart    = %8.4f         detInc = %8.4f\n", m_g.det_start, m_g.det_inc);
  if (m_views.empty()) return;
  const int nView = m_g.n_view;
  if (startView < 0) startView = 0;
  if (endView < 0) endView = nView - 1;
  if (startView > nView - 1) startView = nView - 1;
  if (endView > nView - 1) endView = nView - 1;
  for (int ir = startView; ir <= endView - 1; ir++) {   // the reference stops one short
    std::printf("View %d: angle %f\n", ir, m_views[ir].viewAngle());
    const DetectorValue* v = m_views[ir].detValues();
    for (int id = 0; id < m_g.n_det; id++) std::printf("%8.4f  ", v[id]);
    std::printf("\n");
  }
}

bool Projections::copyHeader(const char* fn, std::ostream& os) {
  std::vector<char> b;
  if (!slurp(fn, b) || b.size() < 4) return false;
  uint16_t hs, sig;
  std::memcpy(&hs, b.data(), 2);
  std::memcpy(&sig, b.data() + 2, 2);
  if (sig != 'P' * 256 + 'J') {
    std::fprintf(stderr, "Illegal signature in projection file %s\n", fn);
    return false;
  }
  if (hs > b.size()) return false;
  os.write(b.data(), hs);
  return (bool)os;
}

bool Projections::copyViewData(const char* fn, std::ostream& os, int startView, int endView) {
  std::vector<char> b;
  if (!slurp(fn, b) || b.size() < 12) {
    std::fprintf(stderr, "Unable to read projection file %s\n", fn);
    return false;
  }
  uint16_t hs, sig;
  uint32_t nv, nd;
  std::memcpy(&hs, b.data(), 2);
  std::memcpy(&sig, b.data() + 2, 2);
  std::memcpy(&nv, b.data() + 4, 4);
  std::memcpy(&nd, b.data() + 8, 4);
  if (sig != 'P' * 256 + 'J') {
    std::fprintf(stderr, "Illegal signature in projection file %s\n", fn);
    return false;
  }
  const int nView = (int)nv;   // projections.cpp:706-717
  if (startView < 0) startView = 0;
  if (startView > nView - 1) startView = nView;
  if (endView < 0 || endView > nView - 1) endView = nView - 1;
  if (startView > endView) std::swap(startView, endView);
  const size_t sizeView = 12 + 4 * (size_t)nd;
  for (int i = startView; i <= endView; i++) {
    const size_t off = hs + (size_t)i * sizeView;
    if (off + sizeView > b.size()) {
      std::fprintf(stderr, "Error reading projection file\n");
      return false;
    }
    os.write(b.data() + off, sizeView);
    if (!os) return false;
  }
  return true;
}

int Projections::convertInterpNameToID(const char* name) {   // projections.cpp:36-50, 90-101
  if (name && !strcasecmp(name, "nearest")) return 0;
  if (name && !strcasecmp(name, "bilinear")) return 1;
  return -1;
}

bool Projections::convertPolar(ImageFile& im, int interpID) const {
  if (im.nx() == 0 || im.ny() == 0 || m_views.empty()) return false;
  const char* name = interpID == 0 ? "nearest" : interpID == 1 ? "bilinear" : nullptr;
  if (!name) return true;   // the reference's interpolatePolar writes nothing then
  const size_t rows = sizeof(float) * (size_t)m_g.n_view * m_pitch;
  float *dS = nullptr, *dI = nullptr;
  bool ok = cudaMalloc(&dS, rows) == cudaSuccess &&
            cudaMalloc(&dI, sizeof(float) * (size_t)im.nx() * im.ny()) == cudaSuccess &&
            cudaMemcpy(dS, m_data.data(), rows, cudaMemcpyHostToDevice) == cudaSuccess;
  std::vector<double> ang = viewAngles();
  if (ok) ok = ctgpu_convert_polar(&m_g, dS, m_pitch, ang.data(), im.nx(), im.ny(), name, dI,
                                   nullptr) == CTGPU_OK;
  if (ok) ok = cudaMemcpy(im.data(), dI, sizeof(float) * (size_t)im.nx() * im.ny(),
                          cudaMemcpyDeviceToHost) == cudaSuccess;
  if (!ok) std::fprintf(stderr, "%s\n", ctgpu_last_error());
  cudaFree(dS);
  cudaFree(dI);
  return ok;
}

static int helical_status(const std::string& msg) {
  // the reference's return codes: 1 not enough data, 2 geometry not supported
  return msg.find("not yet implemented") != std::string::npos ||
                 msg.find("Invalid geometry") != std::string::npos
             ? 2
             : 1;
}

int Projections::Helical180LI(int interpView) {   // projections.cpp:200-358
  int nOut = 0;
  if (ctgpu_helical180li_size(&m_g, m_g.n_view, interpView, &nOut) != CTGPU_OK) {
    std::fprintf(stderr, "%s\n", ctgpu_last_error());
    return helical_status(ctgpu_last_error());
  }
  size_t inBytes = sizeof(float) * (size_t)m_g.n_view * m_pitch;
  size_t outBytes = sizeof(float) * (size_t)nOut * m_pitch;
  float *dIn = nullptr, *dOut = nullptr;
  if (cudaMalloc(&dIn, inBytes) != cudaSuccess || cudaMalloc(&dOut, outBytes) != cudaSuccess) {
    cudaFree(dIn);
    return 1;
  }
  std::vector<double> ang(nOut);
  int rc = cudaMemcpy(dIn, m_data.data(), inBytes, cudaMemcpyHostToDevice) == cudaSuccess
               ? ctgpu_helical180li(&m_g, dIn, m_g.n_view, interpView, dOut, m_pitch, ang.data(),
                                    &nOut, nullptr)
               : CTGPU_ERR_CUDA;
  if (rc == CTGPU_OK) rc = ctgpu_sync(nullptr);
  std::vector<float> out((size_t)nOut * m_pitch);
  if (rc == CTGPU_OK && cudaMemcpy(out.data(), dOut, outBytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = CTGPU_ERR_CUDA;
  cudaFree(dIn);
  cudaFree(dOut);
  if (rc != CTGPU_OK) return 1;
  init(nOut, m_g.n_det);
  m_data.swap(out);
  for (int v = 0; v < nOut; v++) {
    m_views[v].m_detValues = m_data.data() + (size_t)v * m_pitch;
    m_views[v].setViewAngle(ang[v]);
  }
  return 0;
}

int Projections::HalfScanFeather() {   // projections.cpp:369-439
  size_t bytes = sizeof(float) * (size_t)m_g.n_view * m_pitch;
  float* d = nullptr;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return 1;
  int rc = cudaMemcpy(d, m_data.data(), bytes, cudaMemcpyHostToDevice) == cudaSuccess
               ? ctgpu_halfscan_feather(&m_g, d, m_g.n_view, m_pitch, nullptr)
               : CTGPU_ERR_CUDA;
  if (rc == CTGPU_OK) rc = ctgpu_sync(nullptr);
  if (rc == CTGPU_OK && cudaMemcpy(m_data.data(), d, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = CTGPU_ERR_CUDA;
  cudaFree(d);
  if (rc != CTGPU_OK) {
    std::fprintf(stderr, "%s\n", ctgpu_last_error());
    return std::string(ctgpu_last_error()).find("PARALLEL") != std::string::npos ? 2 : 1;
  }
  return 0;
}

bool Phantom::isUnitPulse() const { return !strcasecmp(m_name.c_str(), "unit-pulse"); }

void Phantom::convertToImagefile(ImageFile& im, double viewRatio, int nsample, int) const {
  const int nx = im.nx(), ny = im.ny();
  if (nx < 2 || ny < 2) return;   // phantom.cpp:466-467
  float* d = nullptr;
  double ext[4], inc[2];
  size_t bytes = sizeof(float) * (size_t)nx * ny;
  int rc = CTGPU_ERR_CUDA;
  if (cudaMalloc(&d, bytes) == cudaSuccess)
    rc = ctgpu_phantom_rasterize(m_h, nx, ny, viewRatio, nsample, d, ext, inc, nullptr);
  if (rc == CTGPU_OK) rc = ctgpu_sync(nullptr);
  if (rc == CTGPU_OK && cudaMemcpy(im.data(), d, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = CTGPU_ERR_CUDA;
  cudaFree(d);
  if (rc != CTGPU_OK) {
    std::fprintf(stderr, "convertToImagefile: %s\n", ctgpu_last_error());
    return;
  }
  im.setAxisExtent(ext[0], ext[1], ext[2], ext[3]);
  im.setAxisIncrement(inc[0], inc[1]);
}

Projections* Projections::interpolateToParallel() const {   // projections.cpp:1250-1328
  if (m_g.geometry == CTGPU_GEOMETRY_PARALLEL) return const_cast<Projections*>(this);
  Projections* q = new Projections(m_g.n_view, m_g.n_det);
  size_t inBytes = sizeof(float) * (size_t)m_g.n_view * m_pitch;
  size_t outBytes = sizeof(float) * (size_t)m_g.n_view * q->m_pitch;
  float *dIn = nullptr, *dOut = nullptr;
  std::vector<double> ang = viewAngles(), outAng(m_g.n_view);
  ctgpu_geometry go;
  int rc = CTGPU_ERR_CUDA;
  if (cudaMalloc(&dIn, inBytes) == cudaSuccess && cudaMalloc(&dOut, outBytes) == cudaSuccess &&
      cudaMemcpy(dIn, m_data.data(), inBytes, cudaMemcpyHostToDevice) == cudaSuccess)
    rc = ctgpu_interpolate_to_parallel(&m_g, dIn, m_pitch, ang.data(), dOut, q->m_pitch, &go,
                                       outAng.data(), nullptr);
  if (rc == CTGPU_OK) rc = ctgpu_sync(nullptr);
  if (rc == CTGPU_OK && cudaMemcpy(q->m_data.data(), dOut, outBytes, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = CTGPU_ERR_CUDA;
  cudaFree(dIn);
  cudaFree(dOut);
  if (rc != CTGPU_OK) {
    std::fprintf(stderr, "interpolateToParallel: %s\n", ctgpu_last_error());
    delete q;
    return nullptr;
  }
  q->m_g = go;
  for (int v = 0; v < m_g.n_view; v++) q->m_views[v].setViewAngle(outAng[v]);
  q->m_calcTime = 0;
  q->m_remark = m_remark + "; Interpolate to Parallel";
  return q;
}

// ============================================================== ImageFile ==
ImageFile::ImageFile()
    : m_nx(0), m_ny(0), m_incKnown(false), m_extKnown(false), m_incX(0), m_incY(0), m_minX(0),
      m_maxX(0), m_minY(0), m_maxY(0) {}
ImageFile::ImageFile(int nx, int ny) : ImageFile() { setArraySize(nx, ny); }

void ImageFile::setArraySize(int nx, int ny) {
  m_nx = nx;
  m_ny = ny;
  m_data.assign((size_t)nx * ny, 0.f);
  m_cols.resize(nx);
  for (int i = 0; i < nx; i++) m_cols[i] = m_data.data() + (size_t)i * ny;
}
void ImageFile::arrayDataClear() { std::fill(m_data.begin(), m_data.end(), 0.f); }
void ImageFile::setAxisIncrement(double x, double y) {
  m_incKnown = true;
  m_incX = x;
  m_incY = y;
}
// The reference's Array2dFile::setAxisExtent (array2dfile.cpp:389-397) stores
// only minX and maxY (maxX and minY keep their previous values); files written
// by it carry exactly that, and so do these.
void ImageFile::setAxisExtent(double minX, double maxX, double, double maxY) {
  m_extKnown = true;
  m_minX = minX;
  m_maxY = maxX;
  m_maxY = maxY;
}
void ImageFile::labelAdd(const std::string& label, double calcTime) {
  Label l;
  l.type = 1;   // L_HISTORY
  l.text = label;
  l.calcTime = calcTime;
  now_date(l.date);
  m_labels.push_back(l);
}

bool ImageFile::fileWrite(const char* fn) {   // array2dfile.cpp:443-520, :602-640
  std::string b;
  put<uint16_t>(b, 0);
  put<uint16_t>(b, 'I' * 256 + 'F');
  put<uint16_t>(b, 7);   // PIXEL_FLOAT32
  put<uint16_t>(b, 4);
  put<uint16_t>(b, (uint16_t)m_labels.size());
  put<uint32_t>(b, m_nx);
  put<uint32_t>(b, m_ny);
  put<uint16_t>(b, 1);   // DATA_TYPE_REAL
  put<uint16_t>(b, m_incKnown);
  put<double>(b, m_incX);
  put<double>(b, m_incY);
  put<uint16_t>(b, m_extKnown);
  for (double x : {m_minX, m_maxX, m_minY, m_maxY, 0.0, 1.0}) put<double>(b, x);
  uint16_t hs = (uint16_t)b.size();
  std::memcpy(&b[0], &hs, 2);
  b.append(reinterpret_cast<const char*>(m_data.data()), sizeof(float) * m_data.size());
  for (const Label& l : m_labels) {
    put<uint16_t>(b, (uint16_t)l.type);
    for (int i = 0; i < 6; i++) put<uint16_t>(b, (uint16_t)l.date[i]);
    put<double>(b, l.calcTime);
    put<uint16_t>(b, (uint16_t)l.text.size());
    b += l.text;
  }
  std::ofstream f(fn, std::ios::binary | std::ios::trunc);
  if (!f) return false;
  f.write(b.data(), b.size());
  return (bool)f;
}

bool ImageFile::fileRead(const char* fn) {
  std::vector<char> b;
  if (!slurp(fn, b)) return false;
  size_t off = 0;
  uint16_t hs, sig, pf, ps, nl, dt, ik, ek;
  uint32_t nx, ny;
  if (!get(b, off, hs) || !get(b, off, sig) || !get(b, off, pf) || !get(b, off, ps) ||
      !get(b, off, nl) || !get(b, off, nx) || !get(b, off, ny) || !get(b, off, dt) ||
      !get(b, off, ik) || !get(b, off, m_incX) || !get(b, off, m_incY) || !get(b, off, ek) ||
      !get(b, off, m_minX) || !get(b, off, m_maxX) || !get(b, off, m_minY) || !get(b, off, m_maxY))
    return false;
  if (sig != 'I' * 256 + 'F' || (ps != 4 && ps != 8)) return false;
  setArraySize((int)nx, (int)ny);
  m_incKnown = ik;
  m_extKnown = ek;
  off = hs;
  size_t n = (size_t)nx * ny;
  if (off + n * ps > b.size()) return false;
  for (size_t i = 0; i < n; i++) {
    if (ps == 4) { float v; std::memcpy(&v, b.data() + off + 4 * i, 4); m_data[i] = v; }
    else { double v; std::memcpy(&v, b.data() + off + 8 * i, 8); m_data[i] = (float)v; }
  }
  // labels after the real (and imaginary) planes (array2dfile.cpp:559-595)
  m_labels.clear();
  size_t lo = off + n * ps * (dt == 2 ? 2 : 1);
  for (int i = 0; i < nl; i++) {
    uint16_t h[7], len;
    double ct;
    if (lo + 24 > b.size()) break;
    std::memcpy(h, b.data() + lo, 14);
    std::memcpy(&ct, b.data() + lo + 14, 8);
    std::memcpy(&len, b.data() + lo + 22, 2);
    if (lo + 24 + len > b.size()) break;
    Label l;
    l.type = h[0];
    for (int j = 0; j < 6; j++) l.date[j] = h[1 + j];
    l.calcTime = ct;
    l.text.assign(b.data() + lo + 24, len);
    m_labels.push_back(l);
    lo += 24 + len;
  }
  return true;
}

// device-backed comparison and arithmetic of real images
namespace {
struct DevImages {
  float* p[3] = {nullptr, nullptr, nullptr};
  ~DevImages() {
    for (float* q : p)
      if (q) cudaFree(q);
  }
};
}  // namespace

bool ImageFile::comparativeStatistics(const ImageFile& c, double& d, double& r, double& e) const {
  // imagefile.cpp:188-191: the reference rejects only when both sizes differ
  // (and then reads past the smaller image); both must match here
  if (c.nx() != m_nx || c.ny() != m_ny) {
    std::fprintf(stderr, "Image sizes differ [ImageFile::comparativeStatistics]\n");
    return false;
  }
  if (m_nx == 0 || m_ny == 0) return false;
  const size_t n = (size_t)m_nx * m_ny;
  DevImages dv;
  double dre[3];
  bool ok = cudaMalloc(&dv.p[0], 4 * n) == cudaSuccess && cudaMalloc(&dv.p[1], 4 * n) == cudaSuccess &&
            cudaMemcpy(dv.p[0], m_data.data(), 4 * n, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(dv.p[1], c.m_data.data(), 4 * n, cudaMemcpyHostToDevice) == cudaSuccess &&
            ctgpu_image_compare(dv.p[0], dv.p[1], 1, m_nx, m_ny, n, dre, nullptr) == CTGPU_OK;
  if (!ok) return false;
  d = dre[0];
  r = dre[1];
  e = dre[2];
  return true;
}

bool ImageFile::printComparativeStatistics(const ImageFile& c, std::ostream& os) const {
  double d, r, e;   // imagefile.cpp:243-256
  if (!comparativeStatistics(c, d, r, e)) return false;
  os << "  Normalized root mean squared distance (d): " << d << std::endl;
  os << "      Normalized mean absolute distance (r): " << r << std::endl;
  os << "Worst case distance (2x2 pixel average) (e): " << e << std::endl;
  return true;
}

bool ImageFile::arith(const char* op, const ImageFile& b, ImageFile& out) const {
  if (m_nx != b.nx() || m_ny != b.ny() || m_nx != out.nx() || m_ny != out.ny()) {
    std::fprintf(stderr, "Difference sizes of images [ImageFile::%s]\n", op);
    return false;
  }
  const size_t n = (size_t)m_nx * m_ny;
  if (!n) return true;
  DevImages dv;
  bool ok = cudaMalloc(&dv.p[0], 4 * n) == cudaSuccess && cudaMalloc(&dv.p[1], 4 * n) == cudaSuccess &&
            cudaMalloc(&dv.p[2], 4 * n) == cudaSuccess &&
            cudaMemcpy(dv.p[0], m_data.data(), 4 * n, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(dv.p[1], b.m_data.data(), 4 * n, cudaMemcpyHostToDevice) == cudaSuccess &&
            ctgpu_image_arith(op, dv.p[0], dv.p[1], dv.p[2], n, nullptr) == CTGPU_OK &&
            cudaMemcpy(out.data(), dv.p[2], 4 * n, cudaMemcpyDeviceToHost) == cudaSuccess;
  return ok;
}
bool ImageFile::addImages(const ImageFile& b, ImageFile& out) const { return arith("add", b, out); }
bool ImageFile::subtractImages(const ImageFile& b, ImageFile& out) const {
  return arith("subtract", b, out);
}
bool ImageFile::multiplyImages(const ImageFile& b, ImageFile& out) const {
  return arith("multiply", b, out);
}
bool ImageFile::divideImages(const ImageFile& b, ImageFile& out) const {
  return arith("divide", b, out);
}

void ImageFile::labelsCopy(const ImageFile& f, const char* id) {
  for (const Label& l : f.m_labels) {
    Label c = l;
    c.text = std::string(id ? id : "") + l.text;
    m_labels.push_back(c);
  }
}

// ========================================================== ProcessSignal ==
ProcessSignal::ProcessSignal(const char* filt, const char* method, double, double inc, int n,
                             double param, const char* domain, const char* gen, int zeropad,
                             int interpF, int, int geometry, double fl, double sdl, SGP*)
    : m_h(nullptr), m_n(n), m_fail(false), m_dIn(nullptr), m_dOut(nullptr) {
  if (strcasecmp(domain, "spatial") && strcasecmp(domain, "frequency")) {
    m_fail = true;
    m_failMessage = std::string("Invalid domain name ") + domain;
    return;
  }
  ctgpu_geometry g;
  std::memset(&g, 0, sizeof(g));
  g.geometry = geometry;
  g.n_det = n;
  g.n_view = 1;
  g.det_inc = inc;
  g.view_diameter = 1.0;
  g.focal_length = fl;
  g.source_detector_length = sdl;
  if (ctgpu_recon_create(&g, 1, 1, filt, param, method, zeropad, gen, "linear", interpF, "table",
                         nullptr, &m_h) != CTGPU_OK) {
    m_fail = true;
    m_failMessage = last_err();
    return;
  }
  int pitch = (n + 3) & ~3;
  cudaMalloc(&m_dIn, sizeof(float) * pitch);
  cudaMalloc(&m_dOut, sizeof(float) * pitch);
}
ProcessSignal::~ProcessSignal() {
  ctgpu_recon_destroy(m_h);
  cudaFree(m_dIn);
  cudaFree(m_dOut);
}
void ProcessSignal::filterSignal(const float in[], double out[]) const {
  if (m_fail) return;
  int pitch = (m_n + 3) & ~3;
  std::vector<float> o(m_n);
  cudaMemcpy(m_dIn, in, sizeof(float) * m_n, cudaMemcpyHostToDevice);
  if (ctgpu_recon_filter(m_h, m_dIn, pitch, 1, m_dOut, pitch, nullptr) != CTGPU_OK ||
      ctgpu_sync(nullptr) != CTGPU_OK) {
    std::fprintf(stderr, "filterSignal: %s\n", ctgpu_last_error());
    return;
  }
  cudaMemcpy(o.data(), m_dOut, sizeof(float) * m_n, cudaMemcpyDeviceToHost);
  for (int i = 0; i < m_n; i++) out[i] = o[i];
}

// ========================================================== Backprojector ==
Backprojector::Backprojector(const Projections& proj, ImageFile& im, const char* bp,
                             const char* interp, int interpF, const ReconstructionROI* roi)
    : m_h(nullptr), m_im(im), m_nDet(proj.nDet()), m_dRow(nullptr), m_dImage(nullptr),
      m_fail(false), m_first(true) {
  ctgpu_roi r;
  if (roi) { r.x_min = roi->m_dXMin; r.y_min = roi->m_dYMin; r.x_max = roi->m_dXMax; r.y_max = roi->m_dYMax; }
  if (ctgpu_recon_create(&proj.gpuGeometry(), im.nx(), im.ny(), "abs_bandlimit", -1,
                         "convolution", 1, "direct", interp, interpF, bp, roi ? &r : nullptr,
                         &m_h) != CTGPU_OK) {
    m_fail = true;
    m_failMessage = last_err();
    return;
  }
  double ext[4], inc[2];
  ctgpu_recon_image_axes(m_h, ext, inc);
  im.setAxisIncrement(inc[0], inc[1]);
  im.setAxisExtent(ext[0], ext[1], ext[2], ext[3]);
  im.arrayDataClear();
  cudaMalloc(&m_dRow, sizeof(float) * ((m_nDet + 3) & ~3));
  cudaMalloc(&m_dImage, sizeof(float) * im.nx() * im.ny());
  cudaMemset(m_dImage, 0, sizeof(float) * im.nx() * im.ny());
}
Backprojector::~Backprojector() {
  ctgpu_recon_destroy(m_h);
  cudaFree(m_dRow);
  cudaFree(m_dImage);
}
void Backprojector::BackprojectView(const double* viewData, double viewAngle) {
  if (m_fail) return;
  std::vector<float> row(m_nDet);
  for (int i = 0; i < m_nDet; i++) row[i] = (float)viewData[i];
  cudaMemcpy(m_dRow, row.data(), sizeof(float) * m_nDet, cudaMemcpyHostToDevice);
  if (ctgpu_recon_backproject(m_h, m_dRow, (m_nDet + 3) & ~3, &viewAngle, 1, m_dImage, 1,
                              nullptr) != CTGPU_OK)
    std::fprintf(stderr, "BackprojectView: %s\n", ctgpu_last_error());
}
void Backprojector::PostProcessing() {
  if (m_fail) return;
  ctgpu_recon_postprocess(m_h, m_dImage, nullptr);
  if (ctgpu_sync(nullptr) != CTGPU_OK) std::fprintf(stderr, "PostProcessing: %s\n", ctgpu_last_error());
  cudaMemcpy(m_im.data(), m_dImage, sizeof(float) * m_im.nx() * m_im.ny(), cudaMemcpyDeviceToHost);
}

// ========================================================== Reconstructor ==
Reconstructor::Reconstructor(const Projections& proj, ImageFile& im, const char* filterName,
                             double param, const char* method, int zeropad, const char* gen,
                             const char* interp, int interpF, const char* bp, int,
                             ReconstructionROI* roi, bool rebin, SGP*)
    : m_rebinned(rebin && proj.geometry() != CTGPU_GEOMETRY_PARALLEL ? proj.interpolateToParallel()
                                                                     : nullptr),
      m_proj(m_rebinned ? *m_rebinned : proj), m_im(im), m_h(nullptr), m_dSino(nullptr),
      m_dImage(nullptr), m_fail(false), m_uploaded(false), m_started(false) {
  // reconstruct.cpp:56: rebinToParallel reconstructs interpolateToParallel()
  if (rebin && proj.geometry() != CTGPU_GEOMETRY_PARALLEL && !m_rebinned) {
    m_fail = true;
    m_failMessage = std::string("interpolateToParallel: ") + last_err();
    return;
  }
  ctgpu_roi r;
  if (roi) { r.x_min = roi->m_dXMin; r.y_min = roi->m_dYMin; r.x_max = roi->m_dXMax; r.y_max = roi->m_dYMax; }
  if (ctgpu_recon_create(&proj.gpuGeometry(), im.nx(), im.ny(), filterName, param, method,
                         zeropad, gen, interp, interpF, bp, roi ? &r : nullptr, &m_h) != CTGPU_OK) {
    m_fail = true;
    m_failMessage = last_err();
    return;
  }
  double ext[4], inc[2];
  ctgpu_recon_image_axes(m_h, ext, inc);
  im.setAxisIncrement(inc[0], inc[1]);
  im.setAxisExtent(ext[0], ext[1], ext[2], ext[3]);
  im.arrayDataClear();
  if (cudaMalloc(&m_dSino, sizeof(float) * (size_t)proj.nView() * proj.pitch()) != cudaSuccess ||
      cudaMalloc(&m_dImage, sizeof(float) * im.nx() * im.ny()) != cudaSuccess) {
    m_fail = true;
    m_failMessage = "device allocation failed";
  }
}
Reconstructor::~Reconstructor() {
  delete m_rebinned;
  ctgpu_recon_destroy(m_h);
  cudaFree(m_dSino);
  cudaFree(m_dImage);
}
void Reconstructor::download() {
  if (ctgpu_sync(nullptr) != CTGPU_OK) std::fprintf(stderr, "Reconstructor: %s\n", ctgpu_last_error());
  cudaMemcpy(m_im.data(), m_dImage, sizeof(float) * m_im.nx() * m_im.ny(), cudaMemcpyDeviceToHost);
}
void Reconstructor::reconstructAllViews() {   // reconstruct.cpp:142-147
  reconstructView(0, m_proj.nView());
  postProcessing();
}
void Reconstructor::reconstructView(int start, int count, SGP*, bool bp, double) {
  if (m_fail) return;
  if (count <= 0) count = m_proj.nView() - start;
  if (!bp || count <= 0) return;
  if (!m_uploaded) {
    cudaMemcpy(m_dSino, m_proj.rowData(), sizeof(float) * (size_t)m_proj.nView() * m_proj.pitch(),
               cudaMemcpyHostToDevice);
    m_angles = m_proj.viewAngles();
    m_uploaded = true;
  }
  int rc = ctgpu_recon_run(m_h, m_dSino, m_proj.pitch(), m_angles.data(), start, count, m_dImage,
                           m_started ? CTGPU_RUN_ACCUMULATE : 0, nullptr);
  if (rc != CTGPU_OK) std::fprintf(stderr, "reconstructView: %s\n", ctgpu_last_error());
  m_started = true;
  download();
}
void Reconstructor::postProcessing() {   // reconstruct.cpp:149-153
  if (m_fail || !m_started) return;
  ctgpu_recon_postprocess(m_h, m_dImage, nullptr);
  download();
}
