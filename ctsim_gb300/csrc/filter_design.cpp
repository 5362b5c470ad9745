// filter_design.cpp -- host-side FP64 design of the projection filter.
//
// Builds, once per reconstruction plan, the filter CTSim's ProcessSignal would
// use (its SignalFilter responses, libctsim/filter.cpp:130-584, and the method
// and generation logic of ProcessSignal::init, libctsim/procsignal.cpp:123-442)
// and folds it into the form the GPU applies: a Toeplitz tap vector of length
// 2*nDet-1 plus a per-sample fan pre-weight (procsignal.cpp:551-561).
//   convolution:   taps[n-i+nDet-1] = dx * h[n-i+nDet-1]
//   frequency:     taps[n-i+nDet-1] = c[(n-i) mod N], c[m] = (1/N) sum_k H[k] cos(2 pi k m/N)
// which is exactly the product the reference's O(N^2) "fourier" method and
// FFTW's real transform pair compute for a real, Fourier-ordered H.
#include "filter_design.h"

#include <cmath>
#include <complex>
#include <cstring>
#include <strings.h>
#include <vector>

namespace ctgpu {

namespace {

constexpr double PI = 3.14159265358979323846;
constexpr double TWOPI = 6.28318530717958647692;
constexpr double FEPS = 1.0E-6;

enum FilterId {
  ABS_BANDLIMIT = 0, ABS_G_HAMMING, ABS_HANNING, ABS_COSINE, ABS_SINC, SHEPP,
  BANDLIMIT, SINC, G_HAMMING, HANNING, COSINE, TRIANGLE
};

double sinc1(double x) { return std::fabs(x) > FEPS ? std::sin(x) / x : 1.0; }
double sinc2(double x, double m) { return std::fabs(x) > FEPS ? std::sin(x * m) / x : 1.0; }
double abscos_integral(double u, double w) {
  return std::fabs(u) > FEPS ? (std::cos(u * w) - 1) / (u * u) + w / u * std::sin(u * w)
                             : (w * w / 2);
}

// frequency response (filter.cpp:403-475)
double freq_response(int id, double bw, double u, double param) {
  double au = std::fabs(u), abw = std::fabs(bw);
  bool out = au >= (abw / 2) + FEPS;
  switch (id) {
    case BANDLIMIT: return out ? 0. : 1.;
    case ABS_BANDLIMIT: return out ? 0. : au;
    case TRIANGLE: return out ? 0. : 1 - au / abw;
    case COSINE: return out ? 0. : std::cos(PI * au / abw);
    case ABS_COSINE: return out ? 0. : au * std::cos(PI * au / abw);
    case SINC: return abw * sinc2(PI * abw * au, 1.);
    case ABS_SINC: return out ? 0. : au * abw * sinc2(PI * abw * au, 1.);
    case HANNING: param = 0.5; [[fallthrough]];
    case G_HAMMING: return out ? 0. : param + (1 - param) * std::cos(TWOPI * au / abw);
    case ABS_HANNING: param = 0.5; [[fallthrough]];
    case ABS_G_HAMMING: return out ? 0. : au * (param + (1 - param) * std::cos(TWOPI * au / abw));
    default: return 0.;
  }
}

bool has_analytic_spatial(int id) {
  switch (id) {
    case BANDLIMIT: case TRIANGLE: case COSINE: case G_HAMMING: case HANNING:
    case ABS_BANDLIMIT: case ABS_COSINE: case ABS_G_HAMMING: case ABS_HANNING:
    case SHEPP: case SINC:
      return true;
    default:
      return false;
  }
}

// analytic spatial response (filter.cpp:525-584)
double spatial_analytic(int id, double bw, double x, double param) {
  double u = TWOPI * x, w = bw / 2, b = PI / bw, b2 = TWOPI / bw;
  switch (id) {
    case BANDLIMIT: return bw * sinc2(u * w, 1.0);
    case TRIANGLE: { double t = sinc2(u * w, 1.0); return bw * t * t; }
    case COSINE: return sinc2(b - u, w) + sinc2(b + u, w);
    case HANNING: param = 0.5; [[fallthrough]];
    case G_HAMMING:
      return 2 * param * std::sin(u * w) / u + (1 - param) * (sinc2(b2 - u, w) + sinc2(b2 + u, w));
    case ABS_BANDLIMIT: return 2 * abscos_integral(u, w);
    case ABS_COSINE: return abscos_integral(b - u, w) + abscos_integral(b + u, w);
    case ABS_HANNING: param = 0.5; [[fallthrough]];
    case ABS_G_HAMMING:
      return 2 * param * abscos_integral(u, w) +
             (1 - param) * (abscos_integral(u - b2, w) + abscos_integral(u + b2, w));
    case SHEPP:
      if (std::fabs(u) < 1E-7) return 4. / (PI * bw * bw);
      return std::fabs((2 / bw) * std::sin(u * w)) * sinc2(u * w, 1.) * sinc2(u * w, 1.);
    case SINC: return std::fabs(x) < bw / 2 ? 1. : 0.;
    default: return 0.;
  }
}

// numeric inverse transform by 500-point Simpson integration (filter.cpp:358-381,
// libctsupport/mathfuncs.cpp:37-67)
double spatial_numeric(int id, double bw, double x, double param) {
  const int n = 500;
  double zmin = 0, zmax = (id == TRIANGLE) ? bw : bw / 2;
  double zinc = (zmax - zmin) / (n - 1), z = zmin;
  std::vector<double> q(n);
  for (int i = 0; i < n; i++, z += zinc) q[i] = freq_response(id, bw, z, param) * std::cos(TWOPI * z * x);
  double area = 0, width = (zmax - zmin) / (double)(n - 1);
  int nDiv = (n - 1) / 2;
  for (int i = 1; i <= nDiv; i++) {
    int xr = 2 * i;
    area += (width / 3.0) * (q[xr - 2] + 4.0 * q[xr - 1] + q[xr]);
  }
  if ((n & 1) == 0) area += width * (q[n - 2] + q[n - 1]) / 2;
  return 2 * area;
}

// sampled filter on [fmin, fmax] (SignalFilter::init, filter.cpp:158-229)
std::vector<double> sample_filter(int id, double fmin, double fmax, int n, double bw,
                                  double param, bool spatial) {
  std::vector<double> f(n);
  double inc = (fmax - fmin) / (n - 1);
  if (spatial && id == SHEPP) {
    double a = 2 * bw, c = -4. / (a * a);
    int center = (n - 1) / 2;
    f[center] = 4. / (a * a);
    for (int i = 1; i <= center; i++) f[center + i] = f[center - i] = c / (4 * (i * i) - 1);
    return f;
  }
  double x = fmin;
  for (int i = 0; i < n; i++, x += inc) {
    if (!spatial) f[i] = freq_response(id, bw, x, param);
    else f[i] = has_analytic_spatial(id) ? spatial_analytic(id, bw, x, param)
                                          : spatial_numeric(id, bw, x, param);
  }
  return f;
}

// natural -> Fourier frequency order (include/fourier.h:50-73)
void to_fourier_order(std::vector<double>& v) {
  int n = (int)v.size();
  std::vector<double> t(n);
  if (n % 2) {
    int h = (n - 1) / 2;
    t[0] = v[h];
    for (int i = 0; i < h; i++) t[i + 1] = v[i + 1 + h];
    for (int i = 0; i < h; i++) t[i + h + 1] = v[i];
  } else {
    int h = n / 2;
    t[0] = v[h];
    for (int i = 0; i < h - 1; i++) t[i + 1] = v[i + h + 1];
    for (int i = 0; i < h; i++) t[i + h] = v[i];
  }
  v.swap(t);
}
void to_natural_order(std::vector<double>& v) {
  int n = (int)v.size();
  std::vector<double> t(n);
  if (n % 2) {
    int h = (n - 1) / 2;
    t[h] = v[0];
    for (int i = 0; i < h; i++) t[i + 1 + h] = v[i + 1];
    for (int i = 0; i < h; i++) t[i] = v[i + h + 1];
  } else {
    int h = n / 2;
    t[h] = v[0];
    for (int i = 0; i < h; i++) t[i] = v[i + h];
    for (int i = 0; i < h - 1; i++) t[i + h + 1] = v[i + 1];
  }
  v.swap(t);
}

// sum_j x[j] exp(sign * 2 pi i jk/n) for real x; angles reduced exactly
// through (j*k mod n) so large n stays accurate.  O(n^2) with a cos/sin table.
void real_dft(const std::vector<double>& x, int sign, std::vector<double>& re,
              std::vector<double>& im) {
  int n = (int)x.size();
  std::vector<double> c(n), s(n);
  for (int t = 0; t < n; t++) {
    double a = TWOPI * t / n;
    c[t] = std::cos(a);
    s[t] = sign * std::sin(a);
  }
  re.assign(n, 0.0);
  im.assign(n, 0.0);
  for (int k = 0; k < n; k++) {
    double sr = 0, si = 0;
    long long idx = 0;
    for (int j = 0; j < n; j++) {
      sr += x[j] * c[idx];
      si += x[j] * s[idx];
      idx += k;
      if (idx >= n) idx -= n;
    }
    re[k] = sr;
    im[k] = si;
  }
}

// in-place radix-2 FFT, exp(sign*2 pi i jk/n), n a power of two
void fft_radix2(std::vector<std::complex<double>>& a, int sign) {
  int n = (int)a.size();
  for (int i = 1, j = 0; i < n; i++) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (int len = 2; len <= n; len <<= 1) {
    for (int k = 0; k < len / 2; k++) {
      double ang = sign * TWOPI * k / len;
      std::complex<double> w(std::cos(ang), std::sin(ang));
      for (int i = 0; i < n; i += len) {
        std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
    }
  }
}

// c[m] = (1/N) sum_k H[k] cos(2 pi k m / N)
std::vector<double> circulant_kernel(const std::vector<double>& H) {
  int N = (int)H.size();
  std::vector<double> c(N);
  if ((N & (N - 1)) == 0) {
    std::vector<std::complex<double>> a(N);
    for (int k = 0; k < N; k++) a[k] = H[k];
    fft_radix2(a, +1);
    for (int m = 0; m < N; m++) c[m] = a[m].real() / N;
  } else {
    std::vector<double> re, im;
    real_dft(H, +1, re, im);
    for (int m = 0; m < N; m++) c[m] = re[m] / N;
  }
  return c;
}

int zeropad_points(int n, int zeropad) {   // ProcessSignal::addZeropadFactor (:867-881)
  if (zeropad > 0) {
    double l2 = std::log((double)n) / std::log(2.0);
    int il = (int)std::floor(l2);
    return 1 << (il + zeropad);
  }
  return n;
}

}  // namespace

int filter_id_from_name(const char* name) {
  // the reference's name table is not in ID order (filter.cpp:30-59)
  static const char* names[12] = {"abs_bandlimit", "abs_hamming", "abs_hanning", "abs_cosine",
                                  "shepp", "abs_sinc", "bandlimit", "sinc", "hamming",
                                  "hanning", "cosine", "triangle"};
  for (int i = 0; i < 12; i++)
    if (strcasecmp(name, names[i]) == 0) return i;
  return -1;
}
int filter_method_from_name(const char* name) {   // procsignal.cpp:42-51
  if (!strcasecmp(name, "convolution")) return kMethodConvolution;
  if (!strcasecmp(name, "fourier")) return kMethodFourier;
  if (!strcasecmp(name, "fouier-table")) return kMethodFourierTable;
  if (!strcasecmp(name, "fft")) return kMethodFFT;
  return -1;
}
int filter_generation_from_name(const char* name) {   // procsignal.cpp:68-71
  if (!strcasecmp(name, "direct")) return kGenDirect;
  if (!strcasecmp(name, "inverse-fourier")) return kGenInverseFourier;
  return -1;
}

bool design_filter(const FilterSpec& sp, FilterDesign& out, std::string& err) {
  const int n = sp.nDet;
  if (n < 2) { err = "need at least 2 detectors"; return false; }
  double inc = sp.detInc, bw = sp.bandwidth;
  if (sp.geometry == 2) {   // equilinear: imaginary detector through the origin (:154-158)
    double scale = sp.sdl / sp.focalLength;
    inc /= scale;
    bw *= scale;
  }
  std::vector<double> taps(2 * n - 1, 0.0);
  if (sp.method == kMethodConvolution) {
    const int nf = 2 * (n - 1) + 1;
    std::vector<double> h;
    if (sp.generation == kGenDirect) {
      h = sample_filter(sp.filterId, -inc * (n - 1), inc * (n - 1), nf, bw, sp.param, true);
    } else {
      std::vector<double> fr =
          sample_filter(sp.filterId, -1. / (2 * inc), 1. / (2 * inc), nf, bw, sp.param, false);
      to_fourier_order(fr);
      std::vector<double> re, im;
      real_dft(fr, -1, re, im);   // FORWARD: exp(-i..), divided by n
      h.resize(nf);
      for (int i = 0; i < nf; i++) h[i] = re[i] / nf;
      to_natural_order(h);
      for (int i = 0; i < nf; i++) h[i] /= inc;
    }
    if (sp.geometry == 2) {
      for (auto& v : h) v *= 0.5;
    } else if (sp.geometry == 1) {
      for (int i = 0; i < nf; i++) {
        int k = i - ((nf - 1) / 2);
        double s = 1 / sinc1(k * inc);
        h[i] *= 0.5 * s * s;
      }
    }
    for (int m = 0; m < nf; m++) taps[m] = h[m] * inc;   // convolve(): sum * dx (:672)
    out.nFilterPoints = nf;
  } else {
    if (sp.method == kMethodFFT && sp.interpFactor != 1) {
      err = "preinterpolation (interp_factor != 1) exists only in the reference's FFTW path";
      return false;
    }
    std::vector<double> H;
    if (sp.generation == kGenDirect) {
      int nf = zeropad_points(n, sp.zeropad);
      double fmin = -1. / (2 * inc), fmax = 1. / (2 * inc);
      if (nf % 2 == 0) fmax -= (fmax - fmin) / nf;
      H = sample_filter(sp.filterId, fmin, fmax, nf, bw, sp.param, false);
      if (sp.geometry == 2) {
        for (auto& v : H) v *= 0.5;
      } else if (sp.geometry == 1) {
        for (int i = 0; i < nf; i++) {
          int k = i - ((nf - 1) / 2);
          double s = 1 / sinc1(k * inc);
          H[i] *= 0.5 * s * s;
        }
      }
      to_fourier_order(H);
    } else {
      int nsp = 2 * (n - 1) + 1;
      int nf = nsp;
      if (sp.zeropad > 0) {
        double l2 = std::log((double)nsp) / std::log(2.0);
        int p2 = (int)std::floor(l2);
        if (l2 != std::floor(l2)) p2++;
        p2 += sp.zeropad - 1;
        nf = 1 << p2;
      }
      std::vector<double> s =
          sample_filter(sp.filterId, -inc * (n - 1), inc * (n - 1), nsp, bw, sp.param, true);
      if (sp.geometry == 2) {
        for (auto& v : s) v *= 0.5;
      } else if (sp.geometry == 1) {
        for (int i = 0; i < nsp; i++) {
          int k = i - ((nsp - 1) / 2);
          double sn = std::sin(k * inc);
          sn = std::fabs(sn) < 1E-7 ? 1 : (k * inc) / sn;
          s[i] *= 0.5 * sn * sn;
        }
      }
      s.resize(nf, 0.0);
      std::vector<double> re, im;
      real_dft(s, +1, re, im);   // BACKWARD: exp(+i..), not divided
      H.resize(nf);
      for (int i = 0; i < nf; i++) H[i] = std::hypot(re[i], im[i]) * inc;
    }
    const int N = (int)H.size();
    std::vector<double> c = circulant_kernel(H);
    for (int d = -(n - 1); d <= n - 1; d++) {
      int m = ((d % N) + N) % N;
      taps[d + n - 1] = c[m];
    }
    out.nFilterPoints = N;
  }
  // fan-beam pre-weighting of the input samples (procsignal.cpp:551-561)
  std::vector<double> w(n, 1.0);
  if (sp.geometry == 2) {
    double fl = sp.focalLength;
    for (int i = 0; i < n; i++) {
      int k = i - n / 2;
      w[i] = fl / std::sqrt(fl * fl + k * k * inc * inc);
    }
  } else if (sp.geometry == 1) {
    for (int i = 0; i < n; i++) {
      int k = i - n / 2;
      w[i] = sp.focalLength * std::cos(k * inc);
    }
  }
  out.taps.assign(taps.begin(), taps.end());
  out.taps64 = taps;
  out.weights.assign(w.begin(), w.end());
  return true;
}

// In-place FP64 radix-2 FFT (decimation in time, bit-reversed input order),
// forward sign; n a power of two.
static void fft64(std::vector<std::complex<double>>& a) {
  const size_t n = a.size();
  for (size_t i = 1, j = 0; i < n; i++) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    const double ang = -2.0 * PI / (double)len;
    for (size_t i = 0; i < n; i += len)
      for (size_t k = 0; k < len / 2; k++) {
        const std::complex<double> w(std::cos(ang * k), std::sin(ang * k));
        const std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
  }
}

void filter_spectrum(const FilterDesign& d, int nDet, FilterSpectrum& out) {
  int N = 1;
  while (N < 2 * nDet - 1) N <<= 1;
  std::vector<std::complex<double>> k(N, 0.0);
  for (int m = -(nDet - 1); m < nDet; m++) k[m >= 0 ? m : N + m] = d.taps64[m + nDet - 1];
  fft64(k);
  out.fftN = N;
  out.spectrum.resize(2 * (size_t)N);
  out.twiddle.resize(2 * (size_t)N);
  for (int f = 0; f < N; f++) {
    out.spectrum[2 * f] = (float)(k[f].real() / N);
    out.spectrum[2 * f + 1] = (float)(k[f].imag() / N);
    const double a = -2.0 * PI * (double)f / (double)N;
    out.twiddle[2 * f] = (float)std::cos(a);
    out.twiddle[2 * f + 1] = (float)std::sin(a);
  }
}

}  // namespace ctgpu
