// ctsimtext.cpp -- the phm2pj, pjrec, pjHinterp, pjinfo, phm2if, pj2if and if2
// command-line tools on the GPU library, with the reference's option tables,
// defaults, file formats and exit codes (tools/phm2pj.cpp:33-393,
// tools/pjrec.cpp:31-366, tools/pjHinterp.cpp:32-149, tools/phm2if.cpp,
// tools/pj2if.cpp:33-133, tools/if2.cpp:33-307, tools/ctsimtext.cpp:239-280).
// pj2if and if2 keep the data on the device between the file reads and
// writes (ctgpu_pj_read_device / ctgpu_if_read_device ... _write_device).  Invoked as
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
#include <vector>

#include <cuda_runtime.h>

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
void pjinfo_usage(const char* program) {
  std::cout << "usage: " << base_name(program) << " proj-file [OPTIONS]\n";
  std::cout << "Display projection file information\n\n";
  std::cout << "   --binaryheader  Dump binary header data\n";
  std::cout << "   --binaryviews   Dump binary view data\n";
  std::cout << "   --startview n   Beginning view number to display (default=0)\n";
  std::cout << "   --endview n     Ending view number to display (default=last view)\n";
  std::cout << "   --dump          Print all scan data ASCII format\n";
  std::cout << "   --version       Print version\n";
  std::cout << "   --help          Print this help message\n";
}

int pjinfo_main(int argc, char* const argv[]) {   // tools/pjinfo.cpp:33-151
  enum { O_BINARYHEADER, O_BINARYVIEWS, O_STARTVIEW, O_ENDVIEW, O_DUMP, O_HELP, O_VERSION };
  const struct option options[] = {{"binaryheader", 0, 0, O_BINARYHEADER},
                                   {"binaryviews", 0, 0, O_BINARYVIEWS},
                                   {"startview", 1, 0, O_STARTVIEW},
                                   {"endview", 1, 0, O_ENDVIEW},
                                   {"dump", 0, 0, O_DUMP},
                                   {"help", 0, 0, O_HELP},
                                   {"version", 0, 0, O_VERSION},
                                   {0, 0, 0, 0}};
  bool dump = false, binHeader = false, binViews = false;
  int startView = 0, endView = -1;
  optind = 0;
  while (1) {
    int c = getopt_long(argc, argv, "", options, nullptr);
    if (c == -1) break;
    switch (c) {
      case O_DUMP: dump = true; break;
      case O_BINARYHEADER: binHeader = true; break;
      case O_BINARYVIEWS: binViews = true; break;
      case O_STARTVIEW:
        if (!parse_int(optarg, startView)) {
          std::cerr << "Error setting --startview to %s" << optarg << std::endl;
          pjinfo_usage(argv[0]);
          return 1;
        }
        break;
      case O_ENDVIEW:
        if (!parse_int(optarg, endView)) {
          std::cerr << "Error setting --endview to %s" << optarg << std::endl;
          pjinfo_usage(argv[0]);
          return 1;
        }
        break;
      case O_VERSION: std::cout << "Version 5.2.0 (GB300)" << std::endl; return 0;
      case O_HELP: case '?': pjinfo_usage(argv[0]); return 0;
      default: pjinfo_usage(argv[0]); return 1;
    }
  }
  if (argc - optind != 1) { pjinfo_usage(argv[0]); return 1; }
  const char* name = argv[optind];
  if (binHeader) {
    Projections::copyHeader(name, std::cout);
  } else if (binViews) {
    Projections::copyViewData(name, std::cout, startView, endView);
  } else {
    Projections pj;
    if (!pj.read(name)) {
      std::cerr << "Can not open projection file " << name << std::endl;
      return 1;
    }
    if (dump) {
      pj.printProjectionData(startView, endView);
    } else {
      std::string info;
      pj.printScanInfo(info);
      std::cout << info;
    }
  }
  return 0;
}

// ------------------------------------------------------------------- pj2if --
// device buffers freed on exit
struct DeviceBuffers {
  std::vector<void*> p;
  void* get(size_t bytes) {
    void* q = nullptr;
    if (cudaMalloc(&q, bytes ? bytes : 1) != cudaSuccess) return nullptr;
    p.push_back(q);
    return q;
  }
  ~DeviceBuffers() {
    for (void* q : p) cudaFree(q);
  }
};

void pj2if_usage(const char* program) {
  std::cout << "usage: " << base_name(program) << " in-proj-file out-if-file [OPTIONS]\n";
  std::cout << "Converts a projection file to a imagefile\n\n";
  std::cout << "   --polar     Convert to polar format\n";
  std::cout << "   --verbose   Verbose mode\n";
  std::cout << "   --version   Print version\n";
  std::cout << "   --help      Print this help message\n";
}

int pj2if_main(int argc, char* const argv[]) {
  enum { O_VERBOSE, O_HELP, O_VERSION, O_POLAR };
  const struct option options[] = {{"polar", 0, 0, O_POLAR},     {"verbose", 0, 0, O_VERBOSE},
                                   {"help", 0, 0, O_HELP},       {"version", 0, 0, O_VERSION},
                                   {0, 0, 0, 0}};
  bool verbose = false;
  optind = 0;
  auto t0 = std::chrono::steady_clock::now();
  while (1) {
    int c = getopt_long(argc, argv, "", options, nullptr);
    if (c == -1) break;
    switch (c) {
      case O_VERBOSE: verbose = true; break;
      case O_POLAR: break;   // accepted and unused, as in the reference
      case O_VERSION: std::cout << "Version 5.2.0 (GB300)" << std::endl; return 0;
      case O_HELP: case '?': pj2if_usage(argv[0]); return 0;
      default: pj2if_usage(argv[0]); return 1;
    }
  }
  if (argc - optind != 2) { pj2if_usage(argv[0]); return 1; }
  const char* pjName = argv[optind];
  const char* imName = argv[optind + 1];
  ctgpu_pj_info info;
  std::vector<char> remark(65536);
  if (ctgpu_pj_read_header(pjName, &info, remark.data(), (int)remark.size()) != CTGPU_OK) {
    std::cerr << "Can not open projection file " << pjName << std::endl;
    return 1;
  }
  if (verbose) {
    Projections pj;
    if (pj.read(pjName)) {
      std::string s;
      pj.printScanInfo(s);
      std::cout << s;
    }
  }
  const int nView = info.geometry.n_view, nDet = info.geometry.n_det;
  const int pitch = (nDet + 3) & ~3;
  DeviceBuffers mem;
  float* dSino = static_cast<float*>(mem.get(sizeof(float) * (size_t)nView * pitch));
  double* dAngles = static_cast<double*>(mem.get(sizeof(double) * (size_t)nView));
  float* dImage = static_cast<float*>(mem.get(sizeof(float) * (size_t)nView * nDet));
  if (!dSino || !dAngles || !dImage) {
    std::cerr << "out of device memory\n";
    return 1;
  }
  if (ctgpu_pj_read_device(pjName, dSino, pitch, dAngles, nullptr, nullptr) != CTGPU_OK ||
      ctgpu_sino_to_image(dSino, pitch, nView, nDet, dImage, nullptr) != CTGPU_OK) {
    std::cerr << ctgpu_last_error() << std::endl;
    return 1;
  }
  ctgpu_if_info out;
  std::memset(&out, 0, sizeof(out));
  out.nx = nDet;
  out.ny = nView;
  out.scale_pv = 1.0;
  // the projections' label (projections.cpp:631-634), then the conversion
  ctgpu_if_label labels[2];
  std::memset(labels, 0, sizeof(labels));
  labels[0].type = 1;
  std::memcpy(labels[0].date, info.date, sizeof(info.date));
  labels[0].calc_time = info.calc_time;
  labels[0].text = remark.data();
  labels[0].text_length = info.remark_length;
  labels[1].type = 1;
  labels[1].text = "Conversion from .pj to .if";
  labels[1].calc_time = seconds_since(t0);
  if (ctgpu_if_write_device(imName, &out, labels, 2, dImage, nullptr) != CTGPU_OK) {
    std::cerr << ctgpu_last_error() << std::endl;
    return 1;
  }
  return 0;
}

// --------------------------------------------------------------------- if2 --
void if2_usage(const char* program) {
  std::cout << "usage: " << base_name(program) << " infile1 infile2 outfile [OPTIONS]\n";
  std::cout << "Perform functions on two input image files\n\n";
  std::cout << "     infile1            Name of first input IF file\n";
  std::cout << "     infile2            Name of second input IF file\n";
  std::cout << "     outfile            Name of output Image or Plot file\n";
  std::cout << "     --add              Add images\n";
  std::cout << "     --sub              Subtract image 2 from image 1\n";
  std::cout << "     --mul              Multiply images\n";
  std::cout << "     --comp             Compare images\n";
  std::cout << "     --column-plot n    Plot column\n";
  std::cout << "     --row-plot n       Plot row\n";
  std::cout << "     --verbose          Verbose modem\n";
  std::cout << "     --version          Print version\n";
  std::cout << "     --help             Print this help message\n";
}

// an .if file's labels, with `prefix` before each text (Array2dFile::labelsCopy)
bool copy_labels(const char* fn, const char* prefix, std::vector<std::string>& texts,
                 std::vector<ctgpu_if_label>& out) {
  ctgpu_if_info info;
  if (ctgpu_if_read_header(fn, &info) != CTGPU_OK) return false;
  std::vector<ctgpu_if_label> l(info.n_labels > 0 ? info.n_labels : 1);
  std::vector<char> buf((size_t)info.n_labels * 65536 + 1);
  int n = 0;
  if (ctgpu_if_read_labels(fn, l.data(), info.n_labels, buf.data(), buf.size(), &n) != CTGPU_OK)
    return false;
  for (int i = 0; i < n && i < info.n_labels; i++) {
    texts.push_back(std::string(prefix) + (l[i].text ? l[i].text : ""));
    out.push_back(l[i]);
  }
  return true;
}

int if2_main(int argc, char* const argv[]) {
  enum { O_ADD, O_SUB, O_MUL, O_DIVIDE, O_COMP, O_ROW_PLOT, O_COLUMN_PLOT, O_VERBOSE, O_HELP,
         O_VERSION };
  const struct option options[] = {
      {"add", 0, 0, O_ADD},          {"sub", 0, 0, O_SUB},
      {"multiply", 0, 0, O_MUL},     {"divide", 0, 0, O_DIVIDE},
      {"comp", 0, 0, O_COMP},        {"column-plot", 1, 0, O_COLUMN_PLOT},
      {"row-plot", 1, 0, O_ROW_PLOT}, {"verbose", 0, 0, O_VERBOSE},
      {"help", 0, 0, O_HELP},        {"version", 0, 0, O_VERSION},
      {0, 0, 0, 0}};
  const char* op = nullptr;
  std::string opTitle;
  bool comp = false, imageOut = false, plotOut = false;
  optind = 0;
  auto t0 = std::chrono::steady_clock::now();
  while (1) {
    int c = getopt_long(argc, argv, "", options, nullptr);
    if (c == -1) break;
    switch (c) {
      case O_ADD: op = "add"; opTitle = "Add Images"; imageOut = true; break;
      case O_SUB: op = "subtract"; opTitle = "Subtract Images"; imageOut = true; break;
      case O_MUL: op = "multiply"; opTitle = "Multiply Images"; imageOut = true; break;
      case O_DIVIDE: op = "divide"; opTitle = "Divide Images"; imageOut = true; break;
      case O_ROW_PLOT: case O_COLUMN_PLOT: {
        int v;
        if (!parse_int(optarg, v)) if2_usage(argv[0]);
        plotOut = true;
        break;
      }
      case O_COMP: comp = true; break;
      case O_VERBOSE: break;
      case O_VERSION: std::cout << "Version 5.2.0 (GB300)" << std::endl; return 0;
      case O_HELP: case '?': if2_usage(argv[0]); return 0;
      default: if2_usage(argv[0]); return 1;
    }
  }
  if ((imageOut || plotOut) && optind + 3 != argc) { if2_usage(argv[0]); return 1; }
  if (!(imageOut || plotOut) && optind + 2 != argc) { if2_usage(argv[0]); return 1; }
  const char* in1 = argv[optind];
  const char* in2 = argv[optind + 1];
  ctgpu_if_info h1, h2;
  if (ctgpu_if_read_header(in1, &h1) != CTGPU_OK || ctgpu_if_read_header(in2, &h2) != CTGPU_OK) {
    std::cerr << "Error reading an image" << std::endl;
    return 1;
  }
  if (h1.nx != h2.nx || h1.ny != h2.ny) {
    std::cerr << "Error: Size of image 1 (" << h1.nx << "," << h1.ny << ") and image 2 ("
              << h2.nx << "," << h2.ny << ") do not match" << std::endl;
    return 1;
  }
  if (imageOut && plotOut) {
    std::cerr << "Both Image and Plot output files can not be selected simultaneously" << std::endl;
    return 1;
  }
  if (plotOut) {
    std::cerr << "if2: plot output files are not part of this library" << std::endl;
    return 1;
  }
  const size_t n = (size_t)h1.nx * h1.ny;
  DeviceBuffers mem;
  float* dA = static_cast<float*>(mem.get(sizeof(float) * n));
  float* dB = static_cast<float*>(mem.get(sizeof(float) * n));
  float* dOut = imageOut ? static_cast<float*>(mem.get(sizeof(float) * n)) : nullptr;
  if (!dA || !dB || (imageOut && !dOut)) {
    std::cerr << "out of device memory\n";
    return 1;
  }
  if (ctgpu_if_read_device(in1, dA, nullptr) != CTGPU_OK ||
      ctgpu_if_read_device(in2, dB, nullptr) != CTGPU_OK) {
    std::cerr << "Error reading an image: " << ctgpu_last_error() << std::endl;
    return 1;
  }
  if (op && ctgpu_image_arith(op, dA, dB, dOut, n, nullptr) != CTGPU_OK) {
    std::cerr << ctgpu_last_error() << std::endl;
    return 1;
  }
  if (comp) {
    double dre[3];
    if (ctgpu_image_compare(dA, dB, 1, h1.nx, h1.ny, n, dre, nullptr) != CTGPU_OK) {
      std::cerr << ctgpu_last_error() << std::endl;
      return 1;
    }
    std::cout << "d=" << dre[0] << ", r=" << dre[1] << ", e=" << dre[2] << std::endl;
  }
  if (imageOut) {
    std::vector<std::string> texts;
    std::vector<ctgpu_if_label> labels;
    copy_labels(in1, "if2 file 1: ", texts, labels);
    copy_labels(in2, "if2 file 2: ", texts, labels);
    texts.push_back(opTitle);
    ctgpu_if_label last;
    std::memset(&last, 0, sizeof(last));
    last.type = 1;
    last.calc_time = seconds_since(t0);
    labels.push_back(last);
    for (size_t i = 0; i < labels.size(); i++) {
      labels[i].text = texts[i].c_str();
      labels[i].text_length = (int32_t)texts[i].size();
    }
    ctgpu_if_info out;
    std::memset(&out, 0, sizeof(out));
    out.nx = h1.nx;
    out.ny = h1.ny;
    out.scale_pv = 1.0;
    if (ctgpu_if_write_device(argv[optind + 2], &out, labels.data(), (int)labels.size(), dOut,
                              nullptr) != CTGPU_OK) {
      std::cerr << ctgpu_last_error() << std::endl;
      return 1;
    }
  }
  return 0;
}

int dispatch(int argc, char* argv[]) {
  const char* f = base_name(argv[0]);
  if (!strcasecmp(f, "phm2pj")) return phm2pj_main(argc, argv);
  if (!strcasecmp(f, "pjrec")) return pjrec_main(argc, argv);
  if (!strcasecmp(f, "pjHinterp")) return pjHinterp_main(argc, argv);
  if (!strcasecmp(f, "pjinfo")) return pjinfo_main(argc, argv);
  if (!strcasecmp(f, "phm2if")) return phm2if_main(argc, argv);
  if (!strcasecmp(f, "pj2if")) return pj2if_main(argc, argv);
  if (!strcasecmp(f, "if2")) return if2_main(argc, argv);
  std::cout << "Unknown function name: " << f << "\n"
            << "usage: ctgpu_ctsimtext phm2pj|pjrec|pjHinterp|pjinfo|phm2if|pj2if|if2 args...\n";
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
