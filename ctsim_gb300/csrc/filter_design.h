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
  std::vector<double> taps64;   // the same in FP64
  std::vector<float> weights;   // nDet input pre-weights
  int nFilterPoints = 0;        // length of the reference's filter array
};

// The Toeplitz product as a circular convolution of length fftN (the power of
// two >= 2*nDet-1, so that no lag wraps): spectrum[f] = DFT(kernel)[f] / fftN
// with kernel[m] = taps[m + nDet - 1] for |m| < nDet (negative m at fftN + m),
// and twiddle[m] = exp(-2 pi i m / fftN); both interleaved (re, im), FP64
// computed, FP32 stored.
struct FilterSpectrum {
  int fftN = 0;
  std::vector<float> spectrum;   // 2 * fftN
  std::vector<float> twiddle;    // 2 * fftN
};
void filter_spectrum(const FilterDesign& d, int nDet, FilterSpectrum& out);

int filter_id_from_name(const char* name);
int filter_method_from_name(const char* name);
int filter_generation_from_name(const char* name);
bool design_filter(const FilterSpec& spec, FilterDesign& out, std::string& err);

}  // namespace ctgpu
