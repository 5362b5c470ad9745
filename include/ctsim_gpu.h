// ctsim_gpu.h -- drop-in C++ classes for CTSim's simulate-and-reconstruct path,
// backed by libctgpu.so (C ABI in ctgpu.h).
//
// Same class names, constructor arguments, member functions and error
// convention (constructors never throw; fail() + failMessage()) as CTSim
// 5.2.0's Phantom (include/phantom.h:135-214), Scanner (include/scanner.h:
// 41-180), Projections (include/projections.h:60-228), ImageFile
// (include/imagefile.h:121-244), Reconstructor (include/reconstruct.h:
// 39-78), ProcessSignal (include/procsignal.h:36-176) and Backprojector
// (include/backprojectors.h:40-106), for the members on this path.
// Differences a caller can see:
//   - Projections stores its rows in one contiguous, 16-byte aligned array;
//     getDetectorArray(i) still returns a DetectorArray view of row i.
//   - ImageFile's getArray() returns column pointers into one contiguous
//     column-major array (the reference allocates one block per column).
//   - Backprojector / Reconstructor accumulate the image on the GPU; the
//     ImageFile is brought up to date by postProcessing(), by the end of
//     reconstructView(), and by Backprojector::PostProcessing().
//   - The SGP* / trace plotting arguments are accepted and ignored (no
//     graphics on this path).
#ifndef CTSIM_GPU_H
#define CTSIM_GPU_H

#include <ostream>
#include <string>
#include <vector>

#include "ctgpu.h"

typedef float DetectorValue;       // include/scanner.h:39
typedef float ImageFileValue;      // include/imagefile.h:110-116 (F32Image)
typedef float* ImageFileColumn;
typedef float** ImageFileArray;
class SGP;                         // graphics device; unused

class ImageFile;

class Phantom {
 public:
  Phantom();
  explicit Phantom(const char* phmName);
  ~Phantom();
  bool createFromPhantom(const char* phmName);
  bool createFromFile(const char* fname);
  void addPElem(const char* type, double cx, double cy, double u, double v, double rot,
                double atten);
  bool fail() const { return m_fail; }
  const std::string& failMessage() const { return m_failMessage; }
  const std::string& name() const { return m_name; }
  int nPElem() const;
  double xmin() const;
  double xmax() const;
  double ymin() const;
  double ymax() const;
  double maxAxisLength() const;
  double getDiameterBoundaryCircle() const;   // include/phantom.h:190-194
  bool isUnitPulse() const;                    // composition P_UNIT_PULSE
  // phantom.cpp:455-542: rasterise into im (all columns), on the device
  void convertToImagefile(ImageFile& im, double dViewRatio, int nsample, int trace = 0) const;
  ctgpu_phantom* handle() const { return m_h; }

 private:
  ctgpu_phantom* m_h;
  bool m_fail;
  std::string m_failMessage, m_name;
  Phantom(const Phantom&);
  Phantom& operator=(const Phantom&);
};

class DetectorArray {
 public:
  DetectorArray() : m_detValues(0), m_nDet(0), m_viewAngle(0) {}
  int nDet() const { return m_nDet; }
  double viewAngle() const { return m_viewAngle; }
  DetectorValue* detValues() { return m_detValues; }
  const DetectorValue* detValues() const { return m_detValues; }
  void setViewAngle(double a) { m_viewAngle = a; }

 private:
  friend class Projections;
  DetectorValue* m_detValues;
  int m_nDet;
  double m_viewAngle;
};

class Projections;

class Scanner {
 public:
  static const int GEOMETRY_INVALID = -1;
  static const int GEOMETRY_PARALLEL = 0;
  static const int GEOMETRY_EQUIANGULAR = 1;
  static const int GEOMETRY_EQUILINEAR = 2;

  Scanner(const Phantom& phm, const char* geometryName, int nDet, int nView, int iOffsetView,
          int nSample, double rot_anglen, double dFocalLengthRatio, double dCenterDetectorRatio,
          double dViewRatio, double dScanRatio);
  ~Scanner();
  void collectProjections(Projections& proj, const Phantom& phm, int trace = 0, SGP* = 0);
  void collectProjections(Projections& proj, const Phantom& phm, int iStartView, int iNumViews,
                          int iOffsetView, bool bStoreAtViewPosition, int trace = 0, SGP* = 0);
  void collectProjections(Projections& proj, const Phantom& phm, int iStartView, int iNumViews,
                          int iOffsetView, int iStorageOffset, int trace = 0, SGP* = 0);
  bool fail() const { return m_fail; }
  const std::string& failMessage() const { return m_failMessage; }
  unsigned int nDet() const { return m_g.n_det; }
  unsigned int nView() const { return m_g.n_view; }
  unsigned int offsetView() const { return m_offsetView; }
  unsigned int startView() const { return 0; }
  double rotInc() const { return m_g.rot_inc; }
  double detInc() const { return m_g.det_inc; }
  double detStart() const { return m_g.det_start; }
  double focalLength() const { return m_g.focal_length; }
  double sourceDetectorLength() const { return m_g.source_detector_length; }
  double centerDetectorLength() const { return m_g.source_detector_length - m_g.focal_length; }
  double viewDiameter() const { return m_g.view_diameter; }
  double fanBeamAngle() const { return m_g.fan_beam_angle; }
  int geometry() const { return m_g.geometry; }
  const ctgpu_geometry& gpuGeometry() const { return m_g; }
  static int convertGeometryNameToID(const char* geometryName);
  static const char* convertGeometryIDToName(int idGeometry);

 private:
  ctgpu_scanner* m_h;
  ctgpu_geometry m_g;
  int m_offsetView;
  bool m_fail;
  std::string m_failMessage;
  Scanner(const Scanner&);
  Scanner& operator=(const Scanner&);
};

class Projections {
 public:
  Projections();
  explicit Projections(const Scanner& scanner);
  Projections(int nView, int nDet);
  ~Projections();
  void initFromScanner(const Scanner& scanner);
  bool read(const char* filename);
  bool read(const std::string& filename) { return read(filename.c_str()); }
  bool write(const char* filename);
  bool write(const std::string& filename) { return write(filename.c_str()); }
  int Helical180LI(int interpolation_view);   // 0 ok, 1 not enough data, 2 bad geometry
  int HalfScanFeather();
  // projections.cpp:1250-1328: a new parallel-beam Projections (the caller
  // deletes it), or this object itself for parallel data; null on failure
  Projections* interpolateToParallel() const;
  DetectorArray& getDetectorArray(int iview) { return m_views[iview]; }
  const DetectorArray& getDetectorArray(int iview) const { return m_views[iview]; }
  int nView() const { return m_g.n_view; }
  int nDet() const { return m_g.n_det; }
  int geometry() const { return m_g.geometry; }
  double rotStart() const { return m_g.rot_start; }
  double rotInc() const { return m_g.rot_inc; }
  double detStart() const { return m_g.det_start; }
  double detInc() const { return m_g.det_inc; }
  double viewDiameter() const { return m_g.view_diameter; }
  double focalLength() const { return m_g.focal_length; }
  double sourceDetectorLength() const { return m_g.source_detector_length; }
  double fanBeamAngle() const { return m_g.fan_beam_angle; }
  double phmLen() const { return m_g.view_diameter / 1.414213562373095049; }
  void setPhmLen(double phmLen) { m_g.view_diameter = phmLen * 1.414213562373095049; }
  void setRotInc(double r) { m_g.rot_inc = r; }
  void setDetInc(double d) { m_g.det_inc = d; }
  void setNView(int nView);
  const std::string& remark() const { return m_remark; }
  void setRemark(const std::string& r) { m_remark = r; }
  double calcTime() const { return m_calcTime; }
  void setCalcTime(double t) { m_calcTime = t; }
  void printScanInfo(std::string& out) const;
  // projections.cpp:899-932, pjinfo --dump (prints views start .. end-1, as there)
  void printProjectionData(int startView, int endView) const;
  // projections.cpp:676-772: the raw header / view records of a file
  static bool copyHeader(const char* filename, std::ostream& os);
  static bool copyViewData(const char* filename, std::ostream& os, int startView, int endView);
  // projections.cpp:953-995 on the device: polar image of these projections
  // (interpolateToParallel first for fan beams); interpID from
  // convertInterpNameToID ("nearest" 0, "bilinear" 1)
  bool convertPolar(ImageFile& rIF, int iInterpolationID) const;
  static int convertInterpNameToID(const char* interpName);
  // contiguous storage: row i at rowData() + i * pitch()
  float* rowData() { return m_data.data(); }
  const float* rowData() const { return m_data.data(); }
  int pitch() const { return m_pitch; }
  std::vector<double> viewAngles() const;
  const ctgpu_geometry& gpuGeometry() const { return m_g; }

 private:
  ctgpu_geometry m_g;
  int m_pitch;
  std::vector<float> m_data;
  std::vector<DetectorArray> m_views;
  std::string m_remark, m_filename;
  double m_calcTime;
  int m_date[6];
  void init(int nView, int nDet);
  void stampDate();
};

class ImageFile {
 public:
  ImageFile();
  ImageFile(int nx, int ny);
  void setArraySize(int nx, int ny);
  int nx() const { return m_nx; }
  int ny() const { return m_ny; }
  ImageFileArray getArray() { return m_cols.data(); }
  float* data() { return m_data.data(); }
  const float* data() const { return m_data.data(); }
  void arrayDataClear();
  void setAxisExtent(double minX, double maxX, double minY, double maxY);
  void setAxisIncrement(double incX, double incY);
  void labelAdd(const std::string& label, double calcTime = 0);
  bool fileWrite(const char* filename);
  bool fileWrite(const std::string& f) { return fileWrite(f.c_str()); }
  bool fileRead(const char* filename);
  // imagefile.cpp:186-256 and :378-528 on the device (real FP32 images)
  bool comparativeStatistics(const ImageFile& imComp, double& d, double& r, double& e) const;
  bool printComparativeStatistics(const ImageFile& imComp, std::ostream& os) const;
  bool addImages(const ImageFile& rRHS, ImageFile& result) const;
  bool subtractImages(const ImageFile& rRHS, ImageFile& result) const;
  bool multiplyImages(const ImageFile& rRHS, ImageFile& result) const;
  bool divideImages(const ImageFile& rRHS, ImageFile& result) const;
  // Array2dFile::labelsCopy (array2dfile.cpp:660-672)
  void labelsCopy(const ImageFile& copyFile, const char* idPrefix = 0);
  int getNumLabels() const { return (int)m_labels.size(); }
  std::string labelText(int i) const { return m_labels[i].text; }

 private:
  bool arith(const char* op, const ImageFile& rRHS, ImageFile& result) const;
  int m_nx, m_ny;
  std::vector<float> m_data;
  std::vector<float*> m_cols;
  bool m_incKnown, m_extKnown;
  double m_incX, m_incY, m_minX, m_maxX, m_minY, m_maxY;
  struct Label { int type; std::string text; double calcTime; int date[6]; };
  std::vector<Label> m_labels;
};

struct ReconstructionROI {   // include/reconstruct.h:36-41
  double m_dXMin;
  double m_dYMin;
  double m_dXMax;
  double m_dYMax;
};

class ProcessSignal {
 public:
  ProcessSignal(const char* szFilterName, const char* szFilterMethodName, double dBandwidth,
                double dSignalIncrement, int nSignalPoints, double dFilterParam,
                const char* szDomainName, const char* szFilterGenerationName, int iZeropad,
                int iPreinterpolationFactor, int iTraceLevel, int iGeometry, double dFocalLength,
                double dSourceDetectorLength, SGP* pSGP = 0);
  ~ProcessSignal();
  void filterSignal(const float input[], double output[]) const;
  bool fail() const { return m_fail; }
  const std::string& failMessage() const { return m_failMessage; }

 private:
  ctgpu_recon* m_h;
  int m_n;
  bool m_fail;
  std::string m_failMessage;
  float* m_dIn;
  float* m_dOut;
};

class Backprojector {
 public:
  Backprojector(const Projections& proj, ImageFile& im, const char* backprojName,
                const char* interpName, int interpFactor, const ReconstructionROI* pROI);
  ~Backprojector();
  void BackprojectView(const double* viewData, double viewAngle);
  void PostProcessing();
  bool fail() const { return m_fail; }
  const std::string& failMessage() const { return m_failMessage; }

 private:
  ctgpu_recon* m_h;
  ImageFile& m_im;
  int m_nDet;
  float* m_dRow;
  float* m_dImage;
  bool m_fail, m_first;
  std::string m_failMessage;
};

class Reconstructor {
 public:
  Reconstructor(const Projections& rProj, ImageFile& rIF, const char* filterName,
                double filt_param, const char* filterMethodName, int zeropad,
                const char* filterGenerationName, const char* interpName, int interpFactor,
                const char* backprojectName, int iTrace, ReconstructionROI* pROI = 0,
                bool bRebinToParallel = false, SGP* pSGP = 0);
  ~Reconstructor();
  bool fail() const { return m_fail; }
  const std::string& failMessage() const { return m_failMessage; }
  void reconstructAllViews();
  void reconstructView(int iStartView = 0, int iViewCount = -1, SGP* = 0,
                       bool bBackprojectView = true, double dGraphWidth = 1.);
  void postProcessing();

 private:
  Projections* m_rebinned;    // owned: interpolateToParallel() of the input, or null
  const Projections& m_proj;
  ImageFile& m_im;
  ctgpu_recon* m_h;
  float* m_dSino;
  float* m_dImage;
  bool m_fail, m_uploaded, m_started;
  std::string m_failMessage;
  std::vector<double> m_angles;
  void download();
};

#endif  // CTSIM_GPU_H
