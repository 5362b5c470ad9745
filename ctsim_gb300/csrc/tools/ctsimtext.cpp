// ctsimtext.cpp -- the phm2pj, pjrec, pjHinterp and pjinfo command-line tools on
// the GPU library, with the reference's option tables, defaults, file formats
// and exit codes (tools/phm2pj.cpp:33-393, tools/pjrec.cpp:31-366,
// tools/pjHinterp.cpp:32-149, tools/ctsimtext.cpp:239-280).  Invoked as
// `ctgpu_ctsimtext <function> args...` or through a link named after the
// function.
#include <getopt.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <strings.h>

#include "../../../include/ctsim_gpu.h"

namespace {

const char* base_name(const char* p) {
  const char* s = std::strrchr(p, '/');
  return s ? s + 1 : p;
}

double seconds_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

bool parse_double(const char* s, double& v) {
  char* e = nullptr;
  v = std::strtod(s, &e);
  return e == s + std::strlen(s);
}
bool parse_int(const char* s, int& v) {
  char* e = nullptr;
  v = (int)std::strtol(s, &e, 10);
  return e == s + std::strlen(s);
}

// ------------------------------------------------------------------ phm2pj --
void phm2pj_usage(const char* program) {
  std::cout << "usage: " << base_name(program)
            << " outfile ndet nview [--phantom phantom-name] [--phmfile filename] [OPTIONS]\n"
               "Calculate (projections) through phantom object, either a predefined --phantom or a --phmfile\n\n"
               "     --phantom        herman | shepp-logan | unit-pulse\n"
               "     --phmfile        Get Phantom from phantom file\n"
               "     --desc           Description of raysum\n"
               "     --nray           Number of rays per detector (default = 1)\n"
               "     --rotangle       Angle to rotate view through (fraction of a circle)\n"
               "     --geometry       parallel (default) | equilinear | equiangular\n"
               "     --focal-length   Focal length ratio (default = 2)\n"
               "     --center-detector-length  (default = 2)\n"
               "     --view-ratio     (default = 1)\n"
               "     --scan-ratio     (default = 1)\n"
               "     --offsetview     Initial gantry offset in 'views' (default = 0)\n"
               "     --trace          none | console\n"
               "     --verbose --debug --version --help\n";
}

int phm2pj_main(int argc, char* const argv[]) {
  enum { O_PHANTOM, O_DESC, O_NRAY, O_ROTANGLE, O_PHMFILE, O_GEOMETRY, O_FOCAL_LENGTH,
         O_CENTER_DETECTOR_LENGTH, O_VIEW_RATIO, O_SCAN_RATIO, O_OFFSETVIEW, O_TRACE, O_VERBOSE,
         O_HELP, O_DEBUG, O_VERSION };
  static struct option opts[] = {
      {"phantom", 1, 0, O_PHANTOM}, {"phmfile", 1, 0, O_PHMFILE}, {"desc", 1, 0, O_DESC},
      {"nray", 1, 0, O_NRAY}, {"rotangle", 1, 0, O_ROTANGLE}, {"geometry", 1, 0, O_GEOMETRY},
      {"focal-length", 1, 0, O_FOCAL_LENGTH},
      {"center-detector-length", 1, 0, O_CENTER_DETECTOR_LENGTH},
      {"offsetview", 1, 0, O_OFFSETVIEW}, {"view-ratio", 1, 0, O_VIEW_RATIO},
      {"scan-ratio", 1, 0, O_SCAN_RATIO}, {"trace", 1, 0, O_TRACE}, {"verbose", 0, 0, O_VERBOSE},
      {"help", 0, 0, O_HELP}, {"debug", 0, 0, O_DEBUG}, {"version", 0, 0, O_VERSION},
      {0, 0, 0, 0}};
  auto t0 = std::chrono::steady_clock::now();
  std::string geometry = "parallel", desc, phmName, phmFile;
  int nray = 1, offsetview = 0, verbose = 0;
  double fl = 2., cd = 2., vr = 1., sr = 1., rotangle = -1;
  optind = 0;
  while (true) {
    int c = getopt_long(argc, argv, "", opts, nullptr);
    if (c == -1) break;
    const char* a = optarg;
    switch (c) {
      case O_PHANTOM: phmName = a; break;
      case O_PHMFILE: phmFile = a; break;
      case O_VERBOSE: verbose = 1; break;
      case O_DEBUG: break;
      case O_TRACE:
        if (strcasecmp(a, "none") && strcasecmp(a, "console") && strcasecmp(a, "phantom") &&
            strcasecmp(a, "proj") && strcasecmp(a, "plot") && strcasecmp(a, "clipping")) {
          phm2pj_usage(argv[0]);
          return 1;
        }
        break;
      case O_DESC: desc = a; break;
      case O_ROTANGLE:
        if (!parse_double(a, rotangle)) { std::cerr << "Error setting --rotangle to " << a << std::endl; phm2pj_usage(argv[0]); return 1; }
        break;
      case O_GEOMETRY: geometry = a; break;
      case O_FOCAL_LENGTH:
        if (!parse_double(a, fl)) { std::cerr << "Error setting --focal-length to " << a << std::endl; phm2pj_usage(argv[0]); return 1; }
        break;
      case O_CENTER_DETECTOR_LENGTH:
        if (!parse_double(a, cd)) { std::cerr << "Error setting --center-detector-length to " << a << std::endl; phm2pj_usage(argv[0]); return 1; }
        break;
      case O_VIEW_RATIO:
        if (!parse_double(a, vr)) { std::cerr << "Error setting --view-ratio to " << a << std::endl; phm2pj_usage(argv[0]); return 1; }
        break;
      case O_SCAN_RATIO:
        if (!parse_double(a, sr)) { std::cerr << "Error setting --scan-ratio to " << a << std::endl; phm2pj_usage(argv[0]); return 1; }
        break;
      case O_NRAY:
        if (!parse_int(a, nray)) { std::cerr << "Error setting --nray to " << a << std::endl; phm2pj_usage(argv[0]); return 1; }
        break;
      case O_OFFSETVIEW:
        if (!parse_int(a, offsetview)) { std::cerr << "Error setting --offsetview to " << a << std::endl; phm2pj_usage(argv[0]); return 1; }
        break;
      case O_VERSION: std::cout << "Version: 5.2.0 (GB300)" << std::endl; return 0;
      case O_HELP: case '?': phm2pj_usage(argv[0]); return 0;
      default: phm2pj_usage(argv[0]); return 1;
    }
  }
  if (phmName.empty() && phmFile.empty()) {
    std::cerr << "No phantom defined\n" << std::endl;
    phm2pj_usage(argv[0]);
    return 1;
  }
  if (optind + 3 != argc) { phm2pj_usage(argv[0]); return 1; }
  const char* outfile = argv[optind];
  int ndet, nview;
  if (!parse_int(argv[optind + 1], ndet)) { std::cerr << "Error setting --ndet to " << argv[optind + 1] << std::endl; phm2pj_usage(argv[0]); return 1; }
  if (!parse_int(argv[optind + 2], nview)) { std::cerr << "Error setting --nview to " << argv[optind + 2] << std::endl; phm2pj_usage(argv[0]); return 1; }
  if (rotangle < 0) rotangle = (geometry == "parallel") ? 0.5 : 1.0;
  std::ostringstream d;   // tools/phm2pj.cpp:279-289
  d << "phm2pj: NDet=" << ndet << ", Nview=" << nview << ", NRay=" << nray
    << ", RotAngle=" << rotangle << "OffsetView =" << offsetview << ", Geometry=" << geometry
    << ", ";
  if (!phmFile.empty()) d << "PhantomFile=" << phmFile;
  else d << "Phantom=" << phmName;
  if (!desc.empty()) d << ": " << desc;
  Phantom phm;
  if (!phmName.empty()) {
    phm.createFromPhantom(phmName.c_str());
    if (phm.fail()) {
      std::cout << phm.failMessage() << std::endl << std::endl;
      phm2pj_usage(argv[0]);
      return 1;
    }
  }
  if (!phmFile.empty()) phm.createFromFile(phmFile.c_str());
  Scanner scanner(phm, geometry.c_str(), ndet, nview, offsetview, nray,
                  rotangle * 6.28318530717958647692, fl, cd, vr, sr);
  if (scanner.fail()) {
    std::cout << "Scanner Creation Error: " << scanner.failMessage() << std::endl;
    return 1;
  }
  Projections pj(scanner);
  scanner.collectProjections(pj, phm, 0, nview, offsetview, true, 0);
  pj.setCalcTime(seconds_since(t0));
  pj.setRemark(d.str());
  pj.write(outfile);
  if (verbose) {
    std::string info;
    pj.printScanInfo(info);
    std::cout << info << "  Remark: " << pj.remark() << "\nRun time: " << pj.calcTime()
              << " seconds\n";
  }
  return 0;
}

// ------------------------------------------------------------------- pjrec --
void pjrec_usage(const char* program) {
  std::cout << "usage: " << base_name(program)
            << " raysum-file image-file nx-image ny-image [OPTIONS]\n"
               "Image reconstruction from raysum projections\n"
               "  --interp        nearest | linear (default) | cubic\n"
               "  --preinterpolation-factor  (default = 1)\n"
               "  --filter        abs_bandlimit (default) | abs_sinc | abs_cosine | abs_hamming |\n"
               "                  abs_hanning | shepp | bandlimit | sinc | cosine | triangle |\n"
               "                  hamming | hanning\n"
               "  --filter-method convolution (default) | fourier | fouier-table | fft\n"
               "  --zeropad n     (default = 1)\n"
               "  --filter-generation  direct (default) | inverse-fourier\n"
               "  --backproj      trig | table | diff | idiff (default)\n"
               "  --filter-param  Alpha level for Hamming filter\n"
               "  --trace none|console  --verbose --debug --version --help\n";
}

int pjrec_main(int argc, char* const argv[]) {
  enum { O_INTERP, O_FILTER, O_FILTER_METHOD, O_ZEROPAD, O_FILTER_PARAM, O_FILTER_GENERATION,
         O_BACKPROJ, O_PREINTERPOLATION_FACTOR, O_VERBOSE, O_TRACE, O_HELP, O_DEBUG, O_VERSION };
  static struct option opts[] = {
      {"interp", 1, 0, O_INTERP}, {"preinterpolation-factor", 1, 0, O_PREINTERPOLATION_FACTOR},
      {"filter", 1, 0, O_FILTER}, {"filter-method", 1, 0, O_FILTER_METHOD},
      {"zeropad", 1, 0, O_ZEROPAD}, {"filter-generation", 1, 0, O_FILTER_GENERATION},
      {"filter-param", 1, 0, O_FILTER_PARAM}, {"backproj", 1, 0, O_BACKPROJ},
      {"trace", 1, 0, O_TRACE}, {"debug", 0, 0, O_DEBUG}, {"verbose", 0, 0, O_VERBOSE},
      {"help", 0, 0, O_HELP}, {"version", 0, 0, O_VERSION}, {0, 0, 0, 0}};
  auto t0 = std::chrono::steady_clock::now();
  // defaults: tools/pjrec.cpp:128-137
  bool verbose = false;
  int zeropad = 1, preinterp = 1;
  double param = -1;
  std::string filter = "abs_bandlimit", method = "convolution", gen = "direct", interp = "linear",
              backproj = "idiff";
  optind = 0;
  while (true) {
    int c = getopt_long(argc, argv, "", opts, nullptr);
    if (c == -1) break;
    const char* a = optarg;
    switch (c) {
      case O_INTERP: interp = a; break;
      case O_PREINTERPOLATION_FACTOR: if (!parse_int(a, preinterp)) { pjrec_usage(argv[0]); return 1; } break;
      case O_FILTER: filter = a; break;
      case O_FILTER_METHOD: method = a; break;
      case O_FILTER_GENERATION: gen = a; break;
      case O_FILTER_PARAM: if (!parse_double(a, param)) { pjrec_usage(argv[0]); return 1; } break;
      case O_ZEROPAD: if (!parse_int(a, zeropad)) { pjrec_usage(argv[0]); return 1; } break;
      case O_BACKPROJ: backproj = a; break;
      case O_VERBOSE: verbose = true; break;
      case O_DEBUG: break;
      case O_TRACE:
        if (strcasecmp(a, "none") && strcasecmp(a, "console") && strcasecmp(a, "phantom") &&
            strcasecmp(a, "proj") && strcasecmp(a, "plot") && strcasecmp(a, "clipping")) {
          pjrec_usage(argv[0]);
          return 1;
        }
        break;
      case O_VERSION: std::cout << "Version: 5.2.0 (GB300)" << std::endl; return 0;
      case O_HELP: case '?': pjrec_usage(argv[0]); return 0;
      default: pjrec_usage(argv[0]); return 1;
    }
  }
  if (optind + 4 != argc) { pjrec_usage(argv[0]); return 1; }
  const char* pjFile = argv[optind];
  const char* imFile = argv[optind + 1];
  int nx = (int)std::strtol(argv[optind + 2], nullptr, 10);
  int ny = (int)std::strtol(argv[optind + 3], nullptr, 10);
  std::ostringstream fd, label;
  if (param >= 0) fd << filter << ": alpha=" << param;
  else fd << filter;
  label << "pjrec: " << nx << "x" << ny << ", " << fd.str() << ", " << interp
        << ", preinterpolationFactor=" << preinterp << ", " << backproj;
  Projections pj;
  if (!pj.read(pjFile)) {
    std::fprintf(stderr, "Unable to read projectfile file %s\n", pjFile);
    std::exit(1);
  }
  if (verbose) {
    std::string info;
    pj.printScanInfo(info);
    std::cout << info;
  }
  ImageFile im(nx, ny);
  Reconstructor rec(pj, im, filter.c_str(), param, method.c_str(), zeropad, gen.c_str(),
                    interp.c_str(), preinterp, backproj.c_str(), 0);
  if (rec.fail()) {
    std::cout << rec.failMessage();
    return 1;
  }
  rec.reconstructAllViews();
  double ct = seconds_since(t0);
  im.labelAdd(pj.remark(), pj.calcTime());
  im.labelAdd(label.str(), ct);
  im.fileWrite(imFile);
  if (verbose) std::cout << "Run time: " << ct << " seconds" << std::endl;
  return 0;
}

// --------------------------------------------------------------- pjHinterp --
void pjHinterp_usage(const char* program) {
  std::cout << "usage: " << base_name(program)
            << " projection-file interp-projection-file [OPTIONS]\n"
               "Interpolation of helical data in raw data space\n"
               "  --interpview     view of the interpolation plane (default: pi + fan angle)\n"
               "  --trace none|console  --verbose --debug --version --help\n";
}

int pjHinterp_main(int argc, char* const argv[]) {
  enum { O_INTERPVIEW, O_VERBOSE, O_TRACE, O_HELP, O_DEBUG, O_VERSION };
  static struct option opts[] = {{"interpview", 1, 0, O_INTERPVIEW}, {"trace", 1, 0, O_TRACE},
                                 {"debug", 0, 0, O_DEBUG},          {"verbose", 0, 0, O_VERBOSE},
                                 {"help", 0, 0, O_HELP},            {"version", 0, 0, O_VERSION},
                                 {0, 0, 0, 0}};
  int interpview = -1;
  bool verbose = false;
  optind = 0;
  while (true) {
    int c = getopt_long(argc, argv, "", opts, nullptr);
    if (c == -1) break;
    switch (c) {
      case O_INTERPVIEW:
        if (!parse_int(optarg, interpview)) {
          std::cerr << "Error setting --interpview to " << optarg << std::endl;
          pjHinterp_usage(argv[0]);
          return 1;
        }
        break;
      case O_VERBOSE: verbose = true; break;
      case O_DEBUG: break;
      case O_TRACE: break;
      case O_VERSION: std::cout << "Version 5.2.0 (GB300)" << std::endl; return 0;
      case O_HELP: case '?': pjHinterp_usage(argv[0]); return 0;
      default: pjHinterp_usage(argv[0]); return 1;
    }
  }
  if (optind + 2 != argc) { pjHinterp_usage(argv[0]); return 1; }
  Projections pj;
  if (!pj.read(argv[optind])) {
    std::cerr << "Error reading input file " << argv[optind] << std::endl;
    return 1;
  }
  if (verbose) {
    std::string info;
    pj.printScanInfo(info);
    std::cout << info;
  }
  if (pj.Helical180LI(interpview) != 0) return 1;
  if (pj.HalfScanFeather() != 0) return 1;
  pj.write(argv[optind + 1]);
  return 0;
}

// ------------------------------------------------------------------ phm2if --
// tools/phm2if.cpp: rasterise a phantom (phantom modes; the filter-response
// mode, ImageFile::filterResponse, is not part of this library)
void phm2if_usage(const char* program) {
  std::cout << "phm2if_usage: " << base_name(program) << " outfile nx ny [--phantom phantom-name] [--phmfile filename] [--filter filter-name] [OPTIONS]\n";
  std::cout << "Generates phantom image by rasterizing the phantom\n\n";
  std::cout << "     outfile         Name of output file for image\n";
  std::cout << "     nx              Number of pixels X-axis\n";
  std::cout << "     ny              Number of pixels Y-axis\n";
  std::cout << "     --view-ratio    View diameter to phantom diameter ratio (default = 1)\n";
  std::cout << "     --phantom       Phantom to use for projection\n";
  std::cout << "        herman       Herman head phantom\n";
  std::cout << "        shepp-logan  Shepp-Logan head phantom\n";
  std::cout << "        unit-pulse    Unit pulse phantom\n";
  std::cout << "     --phmfile       Generate Phantom from phantom file\n";
  std::cout << "     --desc          Description of raysum\n";
  std::cout << "     --nsample       Number of samples per axis per pixel (default = 1)\n";
  std::cout << "     --verbose       Verbose mode\n";
  std::cout << "     --help          Print this help message\n";
}

int phm2if_main(int argc, char* const argv[]) {
  enum { O_PHANTOM, O_DESC, O_NSAMPLE, O_FILTER, O_VIEW_RATIO, O_TRACE, O_VERBOSE, O_HELP,
         O_PHMFILE, O_FILTER_DOMAIN, O_FILTER_BW, O_FILTER_PARAM, O_DEBUG, O_VERSION };
  const struct option phm2if_options[] = {
      {"phantom", 1, 0, O_PHANTOM},         {"phmfile", 1, 0, O_PHMFILE},
      {"desc", 1, 0, O_DESC},               {"nsample", 1, 0, O_NSAMPLE},
      {"filter", 1, 0, O_FILTER},           {"filter-domain", 1, 0, O_FILTER_DOMAIN},
      {"filter-bw", 1, 0, O_FILTER_BW},     {"filter-param", 1, 0, O_FILTER_PARAM},
      {"trace", 1, 0, O_TRACE},             {"view-ratio", 1, 0, O_VIEW_RATIO},
      {"verbose", 0, 0, O_VERBOSE},         {"debug", 0, 0, O_DEBUG},
      {"help", 0, 0, O_HELP},               {"version", 0, 0, O_VERSION},
      {0, 0, 0, 0}};
  std::string phmName, phmFile, filterName, desc;
  int nsample = 1;
  double viewRatio = 1.;
  bool verbose = false;
  char* endptr = nullptr;
  optind = 0;
  while (1) {
    int c = getopt_long(argc, argv, "", phm2if_options, nullptr);
    if (c == -1) break;
    switch (c) {
      case O_PHANTOM: phmName = optarg; break;
      case O_PHMFILE: phmFile = optarg; break;
      case O_VERBOSE: verbose = true; break;
      case O_DEBUG: case O_TRACE: case O_FILTER_DOMAIN: case O_FILTER_BW: case O_FILTER_PARAM: break;
      case O_FILTER: filterName = optarg; break;
      case O_DESC: desc = optarg; break;
      case O_VIEW_RATIO:
        viewRatio = strtod(optarg, &endptr);
        if (endptr != optarg + strlen(optarg)) {
          std::cerr << "Error setting --view-ratio to " << optarg << "\n";
          phm2if_usage(argv[0]);
          return 1;
        }
        break;
      case O_NSAMPLE:
        nsample = (int)strtol(optarg, &endptr, 10);
        if (endptr != optarg + strlen(optarg)) {
          std::cerr << "Error setting --nsample to " << optarg << "\n";
          phm2if_usage(argv[0]);
          return 1;
        }
        break;
      case O_VERSION: std::cout << "Version 5.2.0 (GB300)" << std::endl; return 0;
      case O_HELP: case '?': phm2if_usage(argv[0]); return 0;
      default: phm2if_usage(argv[0]); return 1;
    }
  }
  if (phmName == "" && filterName == "" && phmFile == "") {
    std::cerr << "No phantom defined\n" << std::endl;
    phm2if_usage(argv[0]);
    return 1;
  }
  if (optind + 3 != argc) { phm2if_usage(argv[0]); return 1; }
  const char* out = argv[optind];
  int nx = (int)strtol(argv[optind + 1], &endptr, 10);
  if (endptr != argv[optind + 1] + strlen(argv[optind + 1])) { phm2if_usage(argv[0]); return 1; }
  int ny = (int)strtol(argv[optind + 2], &endptr, 10);
  if (endptr != argv[optind + 2] + strlen(argv[optind + 2])) { phm2if_usage(argv[0]); return 1; }
  if (filterName != "" && phmName == "" && phmFile == "") {
    std::cerr << "phm2if --filter (filter-response images) is not part of this library\n";
    return 1;
  }
  auto t0 = std::chrono::steady_clock::now();
  std::ostringstream oss;
  oss << "phm2if: nx=" << nx << ", ny=" << ny << ", viewRatio=" << viewRatio << ", nsample=" << nsample << ", ";
  if (phmFile != "") oss << "phantomFile=" << phmFile;
  else oss << "phantom=" << phmName;
  if (desc != "") oss << ": " << desc;
  Phantom phm;
  if (phmName != "") {
    phm.createFromPhantom(phmName.c_str());
    if (phm.fail()) {
      std::cout << phm.failMessage() << std::endl << std::endl;
      phm2if_usage(argv[0]);
      return 1;
    }
  }
  if (phmFile != "") phm.createFromFile(phmFile.c_str());
  if (verbose) std::cout << "Rasterize Phantom to Image\n" << std::endl;
  ImageFile im(nx, ny);
  if (phm.isUnitPulse()) im.getArray()[nx / 2][ny / 2] = 1.f;
  else phm.convertToImagefile(im, viewRatio, nsample);
  double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  im.labelAdd(oss.str(), t);
  im.fileWrite(out);
  if (verbose) std::cout << "Time to rasterize phantom: " << t << " seconds\n";
  return 0;
}

// ------------------------------------------------------------------ pjinfo --
int pjinfo_main(int argc, char* const argv[]) {
  if (argc < 2) {
    std::cout << "usage: " << base_name(argv[0]) << " projection-file\n";
    return 1;
  }
  Projections pj;
  if (!pj.read(argv[argc - 1])) {
    std::cerr << "Error reading " << argv[argc - 1] << std::endl;
    return 1;
  }
  std::string info;
  pj.printScanInfo(info);
  std::cout << info;
  return 0;
}

int dispatch(int argc, char* argv[]) {
  const char* f = base_name(argv[0]);
  if (!strcasecmp(f, "phm2pj")) return phm2pj_main(argc, argv);
  if (!strcasecmp(f, "pjrec")) return pjrec_main(argc, argv);
  if (!strcasecmp(f, "pjHinterp")) return pjHinterp_main(argc, argv);
  if (!strcasecmp(f, "pjinfo")) return pjinfo_main(argc, argv);
  if (!strcasecmp(f, "phm2if")) return phm2if_main(argc, argv);
  std::cout << "Unknown function name: " << f << "\n"
            << "usage: ctgpu_ctsimtext phm2pj|pjrec|pjHinterp|pjinfo|phm2if args...\n";
  return 1;
}

}  // namespace

int main(int argc, char* argv[]) {
  int rc = 1;
  try {
    const char* self = base_name(argv[0]);
    if (!strcmp(self, "ctgpu_ctsimtext") || !strcmp(self, "ctsimtext")) {
      if (argc < 2) return dispatch(1, argv);
      rc = dispatch(argc - 1, argv + 1);
    } else {
      rc = dispatch(argc, argv);
    }
  } catch (std::exception& e) {
    std::cerr << "Exception: " << e.what() << std::endl;
  } catch (...) {
    std::cerr << "Unknown exception\n";
  }
  return rc;
}
