// filter_design.h -- FP64 host design of the projection filter (see filter_design.cpp).
#pragma once
#include <string>
#include <vector>

namespace ctgpu {

enum { kMethodConvolution = 0, kMethodFourier = 1, kMethodFourierTable = 2, kMethodFFT = 3 };
enum { kGenDirect = 0, kGenInverseFourier = 1 };

struct FilterSpec {
  int filterId, method, generation, zeropad, interpFactor, geometry, nDet;
  double param, bandwidth, detInc, focalLength, sdl;
};

struct FilterDesign {
  std::vector<float> taps;      // 2*nDet-1 Toeplitz taps
  std::vector<float> weights;   // nDet input pre-weights
  int nFilterPoints = 0;        // length of the reference's filter array
};

int filter_id_from_name(const char* name);
int filter_method_from_name(const char* name);
int filter_generation_from_name(const char* name);
bool design_filter(const FilterSpec& spec, FilterDesign& out, std::string& err);

}  // namespace ctgpu
