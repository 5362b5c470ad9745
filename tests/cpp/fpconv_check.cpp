// Checks the integer-pipe FP32 <-> FP64 conversions of
// ctsim_gb300/csrc/k_fpconv.cuh (host build of the same code the kernels use)
// against this CPU's own conversions (IEEE 754, round to nearest even), bit
// for bit: every float exponent with random fractions, ties constructed at
// every exponent, the edges of the float range, zeros, subnormals, infinities
// and NaNs.  Prints the number of cases and exits 1 on the first mismatch.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

#include "../../ctsim_gb300/csrc/k_fpconv.cuh"

using namespace ctgpu;

static uint64_t bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static uint32_t bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static double dbl(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static float flt(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static long cases = 0;

static bool same_f(float a, float b) {
  if (std::isnan(a) && std::isnan(b)) return true;
  return bits(a) == bits(b);
}
static bool same_d(double a, double b) {
  if (std::isnan(a) && std::isnan(b)) return true;
  return bits(a) == bits(b);
}

static bool check_d(double d) {
  cases++;
  volatile double v = d;
  const float want = (float)v, got = f64_to_f32_rn(d);
  if (!same_f(want, got)) {
    std::printf("f64_to_f32_rn(%016llx): %08x, want %08x\n", (unsigned long long)bits(d),
                bits(got), bits(want));
    return false;
  }
  const double wz = v + 0.0, gz = plus_zero(d);
  if (!same_d(wz, gz)) {
    std::printf("plus_zero(%016llx)\n", (unsigned long long)bits(d));
    return false;
  }
  return true;
}
static bool check_f(float f) {
  cases++;
  volatile float v = f;
  const double want = (double)v, got = f32_to_f64(f);
  if (!same_d(want, got)) {
    std::printf("f32_to_f64(%08x): %016llx, want %016llx\n", bits(f),
                (unsigned long long)bits(got), (unsigned long long)bits(want));
    return false;
  }
  return true;
}

int main() {
  std::mt19937_64 rng(20261204);
  // floats: every exponent (subnormals and specials included), both signs
  for (uint32_t e = 0; e < 256; e++)
    for (int k = 0; k < 4000; k++) {
      const uint32_t u = (uint32_t)(rng() & 0x807FFFFFu) | (e << 23);
      if (!check_f(flt(u))) return 1;
    }
  for (uint32_t u : {0u, 0x80000000u, 1u, 0x807FFFFFu, 0x7F7FFFFFu, 0x7F800000u, 0xFF800000u,
                     0x7FC00000u, 0x00800000u})
    if (!check_f(flt(u))) return 1;
  // doubles around and across the float range, random fractions
  for (int e = 700; e <= 1300; e++)
    for (int k = 0; k < 2000; k++) {
      const uint64_t u = (rng() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)e << 52);
      if (!check_d(dbl(u))) return 1;
    }
  // ties and near-ties at every exponent of the float range: the 29 dropped
  // bits exactly half, half +- 1, and the kept fraction odd and even
  for (int e = 860; e <= 1160; e++)
    for (int k = 0; k < 400; k++) {
      const uint64_t keep = (rng() & 0x7FFFFFull) << 29;
      for (uint64_t rest : {0x10000000ull, 0x0FFFFFFFull, 0x10000001ull, 0ull, 0x1FFFFFFFull})
        for (uint64_t odd : {0ull, 1ull << 29})
          for (uint64_t sign : {0ull, 1ull << 63}) {
            const uint64_t u = sign | ((uint64_t)e << 52) | ((keep & ~(1ull << 29)) | odd) | rest;
            if (!check_d(dbl(u))) return 1;
          }
    }
  // the largest float, the step to infinity, zeros, subnormal doubles, specials
  const double fmax = (double)std::numeric_limits<float>::max();
  for (double d : {fmax, std::nextafter(fmax, 1e300), fmax + std::ldexp(1.0, 103),
                   fmax + std::ldexp(1.0, 103) - std::ldexp(1.0, 50), -fmax, 0.0, -0.0,
                   std::ldexp(1.0, -1074), -std::ldexp(1.0, -1022), std::ldexp(1.0, -126),
                   std::ldexp(1.0, -127), std::ldexp(1.0, -149), std::ldexp(1.5, -150),
                   std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                   std::numeric_limits<double>::quiet_NaN(), 1.0, -1.0})
    if (!check_d(d)) return 1;
  std::printf("%ld cases\n", cases);
  return 0;
}
