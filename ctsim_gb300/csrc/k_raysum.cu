// k_raysum.cu -- analytic phantom ray-sums on sm_103a.
//
// Computes what Scanner::collectProjections does (libctsim/scanner.cpp:295-533):
// for every detector of every view, nSample rays from the detector sub-cell to
// the source, each summing chord length x attenuation over the phantom's
// elements (projectSingleLine / projectLineAgainstPElem, :611-656), with the
// element's outline bounding box pre-rejecting rays as clipLineWorldCoords
// does (libctsim/phantom.cpp:830-850).
//
// Numerical design (FP32 per ray-element pair, FP64 per view-element setup):
// the chord through an element is a function of the signed distance rho from
// the element centre to the ray and of the ray direction in the element
// frame.  rho is the small difference of large numbers when formed from ray
// end points, so each CTA first solves, in FP64 and once per (view, element),
// for the ray index t_c at which rho vanishes; rho of ray t is then formed as
// slope * (t - t_c) from the exact integer t and the split (int, frac) root,
// which keeps its relative error at FP32 rounding even near tangency.  For the
// equiangular arc the numerator is a difference of sines, rewritten as
// 2 cos(.) sin((alpha_c - alpha_t)/2) with a small, accurately formed argument.
// The pre-rejection box is tested in FP32 with a margin; rays within the
// margin of the box boundary repeat the reference's FP64 Cohen-Sutherland test.
//
// One CTA per view: the per-view FP64 setup is paid once per view.
#include "ctgpu_internal.h"

namespace ctgpu {

namespace {

struct ElemView {
  float kB;          // rho = kB * (t - t_c)   (times 1/|r| for fan beams)
  float tcF;         // t_c = tcI + tcF
  int tcI;
  int type;
  float ca, sa;      // element rotation
  float u, v, atten;
  float dcbx, dcby;  // outline box centre minus element centre
  float hx, hy, rbox;
  float cpsi, spsi;  // equiangular: cos/sin of psi'
  float ra, rb;      // parallel: ray direction in the element frame
  int live;          // 0: no ray of this view can meet the element
  float rin;         // radius of the outline box's inscribed circle, less the margin
};
static_assert(sizeof(ElemView) % 16 == 0, "ElemView records keep 16-byte alignment");

// byte offset of the per-sub-sample direction table after the element records
__host__ __device__ inline size_t dir_table_offset(int nRecords) {
  return ((size_t)nRecords * sizeof(ElemView) + 15) & ~(size_t)15;
}

__device__ __forceinline__ double cross2(double ax, double ay, double bx, double by) {
  return ax * by - ay * bx;
}

// sin(x) for |x| <= 1.7 by its Taylor series to x^15 (relative error < 2e-9).
__device__ __forceinline__ float sin_series(float x) {
  float x2 = x * x;
  float p = -1.0f / 1307674368000.0f;
  p = fmaf(p, x2, 1.0f / 6227020800.0f);
  p = fmaf(p, x2, -1.0f / 39916800.0f);
  p = fmaf(p, x2, 1.0f / 362880.0f);
  p = fmaf(p, x2, -1.0f / 5040.0f);
  p = fmaf(p, x2, 1.0f / 120.0f);
  p = fmaf(p, x2, -1.0f / 6.0f);
  return fmaf(p * x2, x, x);
}

// Liang-Barsky step for the constraint n.(P + t r) <= k.
__device__ __forceinline__ void clip_hp(float nx, float ny, float k, float px, float py, float rx,
                                        float ry, float& lo, float& hi) {
  float a = nx * rx + ny * ry;
  float b = k - (nx * px + ny * py);
  if (a > 0.f) hi = fminf(hi, __fdiv_rn(b, a));
  else if (a < 0.f) lo = fmaxf(lo, __fdiv_rn(b, a));
  else if (b < 0.f) { lo = 1.f; hi = 0.f; }
}

// sqrt((r-|s|)(r+|s|)) or 0
__device__ __forceinline__ float half_chord(float r, float s) {
  float as = fabsf(s);
  if (as >= r) return 0.f;
  return sqrtf((r - as) * (r + as));
}

// Chord of the line {P + t (ra,rb)} (element frame, unit direction) with the
// element; P is the foot of the perpendicular from the element centre at
// signed distance rho.
__device__ float element_chord(const ElemView& e, float rho, float ra, float rb) {
  float u = e.u, v = e.v;
  if (e.type == kEllipse) {
    float xa = ra / u, xb = rb / v;
    float E = fmaf(xa, xa, xb * xb);
    float uv = u * v;
    float h = uv * sqrtf(E);
    float hc = half_chord(h, rho);
    return hc == 0.f ? 0.f : __fdividef(2.f * hc, E * uv);
  }
  float px = rho * rb, py = -rho * ra;
  float lo = -INFINITY, hi = INFINITY;
  if (e.type == kRect) {
    clip_hp(1.f, 0.f, u, px, py, ra, rb, lo, hi);
    clip_hp(-1.f, 0.f, u, px, py, ra, rb, lo, hi);
    clip_hp(0.f, 1.f, v, px, py, ra, rb, lo, hi);
    clip_hp(0.f, -1.f, v, px, py, ra, rb, lo, hi);
  } else if (e.type == kTriangle) {
    clip_hp(0.f, -1.f, 0.f, px, py, ra, rb, lo, hi);
    clip_hp(1.f / u, 1.f / v, 1.f, px, py, ra, rb, lo, hi);
    clip_hp(-1.f / u, 1.f / v, 1.f, px, py, ra, rb, lo, hi);
  } else {   // segment / sector: circle centred (0, v), radius sqrt(u^2+v^2)
    float R = sqrtf(fmaf(u, u, v * v));
    float sc = fmaf(v, ra, rho);
    float hc = half_chord(R, sc);
    if (hc == 0.f) return 0.f;
    float tc = v * rb;
    lo = tc - hc;
    hi = tc + hc;
    if (e.type == kSegment) {
      clip_hp(0.f, 1.f, 0.f, px, py, ra, rb, lo, hi);
    } else {
      float m = v / u;
      clip_hp(m, 1.f, v, px, py, ra, rb, lo, hi);
      clip_hp(-m, 1.f, v, px, py, ra, rb, lo, hi);
    }
  }
  return hi > lo ? hi - lo : 0.f;
}

// Cohen-Sutherland region code / clip, FP64 (libctsupport/clip.cpp:331-395).
__device__ int rect_code(double x, double y, const double r[4]) {
  int c = 0;
  if (x < r[0]) c = 1;
  else if (x > r[2]) c = 2;
  if (y < r[1]) c += 4;
  else if (y > r[3]) c += 8;
  return c;
}
__device__ bool clip_rect_fp64(double x1, double y1, double x2, double y2, const double r[4]) {
  int c1 = rect_code(x1, y1, r), c2 = rect_code(x2, y2, r);
  for (int guard = 0; guard < 16 && (c1 || c2); guard++) {
    if (c1 & c2) return false;
    int c = c1 ? c1 : c2;
    double x = 0, y = 0;
    if (c & 1) { y = y1 + (y2 - y1) * (r[0] - x1) / (x2 - x1); x = r[0]; }
    else if (c & 2) { y = y1 + (y2 - y1) * (r[2] - x1) / (x2 - x1); x = r[2]; }
    else if (c & 4) { x = x1 + (x2 - x1) * (r[1] - y1) / (y2 - y1); y = r[1]; }
    else if (c & 8) { x = x1 + (x2 - x1) * (r[3] - y1) / (y2 - y1); y = r[3]; }
    if (c == c1) { x1 = x; y1 = y; c1 = rect_code(x1, y1, r); }
    else { x2 = x; y2 = y; c2 = rect_code(x2, y2, r); }
  }
  return true;
}

// FP32 test of the infinite ray line against the element's outline box:
// +1 clearly hits, -1 clearly misses, 0 within the rounding margin.
__device__ __forceinline__ int box_test(const ElemView& e, float rho, float rx, float ry) {
  float rhob = rho + (rx * e.dcby - ry * e.dcbx);
  float px = rhob * ry, py = -rhob * rx;   // foot from the box centre (world frame)
  float margin = 1e-5f * (e.hx + e.hy) + 1e-9f;
  float lo = -INFINITY, hi = INFINITY;
  bool amb = false;
  // x slabs
  if (fabsf(rx) > 0.f) {
    float t1 = __fdiv_rn(-e.hx - px, rx), t2 = __fdiv_rn(e.hx - px, rx);
    lo = fmaxf(lo, fminf(t1, t2));
    hi = fminf(hi, fmaxf(t1, t2));
  } else {
    float b = e.hx - fabsf(px);
    if (b < -margin) return -1;
    if (b <= margin) amb = true;
  }
  if (fabsf(ry) > 0.f) {
    float t1 = __fdiv_rn(-e.hy - py, ry), t2 = __fdiv_rn(e.hy - py, ry);
    lo = fmaxf(lo, fminf(t1, t2));
    hi = fminf(hi, fmaxf(t1, t2));
  } else {
    float b = e.hy - fabsf(py);
    if (b < -margin) return -1;
    if (b <= margin) amb = true;
  }
  float gap = hi - lo;
  if (gap < -margin) return -1;
  if (amb || gap <= margin) return 0;
  return 1;
}

struct ViewGeom {   // FP64 per-view quantities shared by the setup and the rays
  double S0x, S0y, dSx, dSy;       // source (parallel: per detector step)
  double D0x, D0y, dDx, dDy;       // detector point of ray 0 and per-ray step
  double dDetx, dDety;             // parallel: per-detector detector step
  double alpha0, delta;            // equiangular arc: angle of ray 0, step
};

template <int GEOM>
__device__ void view_geom(const RaysumLaunch& L, const ViewPos& vp, ViewGeom& g) {
  int nDet = L.nDet, nS = L.nSample;
  double sdx = (vp.xs2 - vp.xs1) / nDet, sdy = (vp.ys2 - vp.ys1) / nDet;
  g.S0x = vp.xs1 + sdx / 2;
  g.S0y = vp.ys1 + sdy / 2;
  g.dSx = sdx;
  g.dSy = sdy;
  if (GEOM == kEquiangular) {
    g.delta = L.angularDetInc / nS;
    g.alpha0 = vp.angle + 3 * kHalfPi - (L.angularDetLen / 2) + g.delta / 2;
  } else {
    double ddx = (vp.xd2 - vp.xd1) / nDet, ddy = (vp.yd2 - vp.yd1) / nDet;
    double ddx2 = ddx / nS, ddy2 = ddy / nS;
    g.D0x = vp.xd1 + ddx2 / 2;
    g.D0y = vp.yd1 + ddy2 / 2;
    g.dDx = ddx2;
    g.dDy = ddy2;
    g.dDetx = ddx;
    g.dDety = ddy;
  }
}

__device__ __forceinline__ void split_root(double t, int& ti, float& tf) {
  double fl = floor(t);
  if (fl > 2.0e9) fl = 2.0e9;
  if (fl < -2.0e9) fl = -2.0e9;
  ti = (int)fl;
  tf = (float)(t - fl);
}

// Per-view FP64 quantities of the equiangular set-up shared by all elements:
// unit vectors of the first ray's arc angle alpha0 and of the arc's middle,
// and mid - alpha0.
struct ArcFrame {
  double c0, s0, cm, sm, midRel, invDelta;
};

template <int GEOM>
__device__ void setup_element(const RaysumLaunch& L, const ViewGeom& g, const ArcFrame& af,
                              const PElem& pe, int sub, ElemView& e) {
  e.type = pe.type;
  e.ca = (float)pe.cosr;
  e.sa = (float)pe.sinr;
  e.u = (float)pe.u;
  e.v = (float)pe.v;
  e.atten = (float)pe.atten;
  e.dcbx = pe.dcbx;
  e.dcby = pe.dcby;
  e.hx = pe.hx;
  e.hy = pe.hy;
  e.rbox = pe.rbox;
  e.rin = pe.rin;
  e.live = 1;
  e.cpsi = e.spsi = 0.f;
  e.ra = e.rb = 0.f;
  if (GEOM == kParallel) {
    // ray direction of sub-sample `sub` (independent of the detector index)
    double rx = (g.D0x + sub * g.dDx) - g.S0x, ry = (g.D0y + sub * g.dDy) - g.S0y;
    double inv = 1.0 / sqrt(rx * rx + ry * ry);
    rx *= inv;
    ry *= inv;
    double wx = pe.cx - g.S0x, wy = pe.cy - g.S0y;
    double A = cross2(rx, ry, wx, wy), B = cross2(rx, ry, g.dSx, g.dSy);
    // rho(d) = A - d B
    if (B == 0.0) { e.live = 0; return; }
    split_root(A / B, e.tcI, e.tcF);
    e.kB = (float)(-B);
    e.ra = (float)(rx * pe.cosr + ry * pe.sinr);
    e.rb = (float)(-rx * pe.sinr + ry * pe.cosr);
  } else if (GEOM == kEquilinear) {
    double wx = pe.cx - g.S0x, wy = pe.cy - g.S0y;
    double A = cross2(g.D0x - g.S0x, g.D0y - g.S0y, wx, wy);
    double B = cross2(g.dDx, g.dDy, wx, wy);
    if (B == 0.0) { e.live = 0; return; }
    split_root(-A / B, e.tcI, e.tcF);
    e.kB = (float)B;
  } else {
    // The arc point D(a) = CD (cos a, sin a) sees the element centre W from the
    // source S when cross(D(a) - S, W - S) = 0, i.e. sin(theta_w - a) = q with
    // w = W - S, theta_w its angle and q = cross(S, w) / (CD |w|).  The two
    // solutions a = theta_w - b and theta_w - pi + b (sin b = q) have the unit
    // vectors R(-b) w/|w| and -R(b) w/|w|; the one nearer the arc's middle is
    // taken, and its angle is measured from the middle (atan2 in (-pi, pi]),
    // which is the reference's branch choice without an arcsine.
    const double CD = L.centerDetectorLength;
    const double wx = pe.cx - g.S0x, wy = pe.cy - g.S0y;
    const double wn = sqrt(wx * wx + wy * wy);
    const double q = cross2(g.S0x, g.S0y, wx, wy) / (CD * wn);
    if (!(fabs(q) <= 1.0)) { e.live = 0; return; }
    const double cb = sqrt((1.0 - q) * (1.0 + q));
    const double iw = 1.0 / wn;
    const double u1x = (wx * cb + wy * q) * iw, u1y = (wy * cb - wx * q) * iw;
    const double u2x = -(wx * cb - wy * q) * iw, u2y = -(wy * cb + wx * q) * iw;
    const double d1 = u1x * af.cm + u1y * af.sm, d2 = u2x * af.cm + u2y * af.sm;
    const double ux = d1 >= d2 ? u1x : u2x, uy = d1 >= d2 ? u1y : u2y;
    const double rel = atan2(af.cm * uy - af.sm * ux, af.cm * ux + af.sm * uy) + af.midRel;
    split_root(rel * af.invDelta, e.tcI, e.tcF);
    e.kB = (float)(2.0 * CD * wn);
    // psi = theta_w - (a + alpha0)/2 = (theta_w - alpha0) - rel/2 enters only
    // through its cosine and sine: FP32
    const float thw0 = atan2f((float)(af.c0 * wy - af.s0 * wx), (float)(af.c0 * wx + af.s0 * wy));
    float sp, cp;
    sincosf(thw0 - 0.5f * (float)rel, &sp, &cp);
    e.cpsi = cp;
    e.spsi = sp;
  }
}

}  // namespace

// per-view values, computed once per CTA by one thread (FP64 is 1/64 of the
// FP32 rate on this GPU)
struct ViewShared {
  ViewGeom g;
  ArcFrame af;
  double ca0, sa0;
};

template <int GEOM>
__global__ void __launch_bounds__(128) raysum_kernel(RaysumLaunch L) {
  extern __shared__ __align__(16) ElemView ev[];
  __shared__ ViewShared vs;
  const int view = blockIdx.x;
  const int nS = L.nSample;
  const int nSub = (GEOM == kParallel) ? nS : 1;
  const PElem* elems = L.elems;
  int nElem = L.nElem;
  float* sino = L.sino + (size_t)blockIdx.y * L.sliceStride;
  if (L.elemOffset) {
    elems += L.elemOffset[blockIdx.y];
    nElem = L.elemOffset[blockIdx.y + 1] - L.elemOffset[blockIdx.y];
  }
  if (threadIdx.x == 0) {
    const ViewPos vp = L.views[view];
    view_geom<GEOM>(L, vp, vs.g);
    vs.af = ArcFrame{};
    vs.ca0 = 1.0;
    vs.sa0 = 0.0;
    if (GEOM == kEquiangular) {
      const double mid = vs.g.alpha0 + 0.5 * (L.nDet * L.nSample - 1) * vs.g.delta;
      sincos(vs.g.alpha0, &vs.af.s0, &vs.af.c0);
      sincos(mid, &vs.af.sm, &vs.af.cm);
      vs.af.midRel = mid - vs.g.alpha0;
      vs.af.invDelta = 1.0 / vs.g.delta;
      vs.ca0 = vs.af.c0;
      vs.sa0 = vs.af.s0;
    }
  }
  __syncthreads();
  const ViewGeom& g = vs.g;
  float2* sdir = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(ev) +
                                           dir_table_offset(L.nElem * nSub));   // per sub-sample
  for (int k = threadIdx.x; k < nElem * nSub; k += blockDim.x)
    setup_element<GEOM>(L, g, vs.af, elems[k / nSub], k % nSub, ev[k]);
  if (GEOM == kParallel) {
    for (int i = threadIdx.x; i < nS; i += blockDim.x) {
      double drx = (g.D0x + i * g.dDx) - g.S0x, dry = (g.D0y + i * g.dDy) - g.S0y;
      double inv = 1.0 / sqrt(drx * drx + dry * dry);
      sdir[i] = make_float2((float)(drx * inv), (float)(dry * inv));
    }
  }
  __syncthreads();

  // FP32 copies of the per-ray affine quantities
  const float rsx = (float)(g.D0x - g.S0x), rsy = (float)(g.D0y - g.S0y);
  const float stx = (float)g.dDx, sty = (float)g.dDy;
  const float hdelta = (float)(0.5 * g.delta);
  const float fca0 = (float)vs.ca0, fsa0 = (float)vs.sa0;
  const float CD = (float)L.centerDetectorLength;
  const float Sx = (float)g.S0x, Sy = (float)g.S0y;

  for (int d = threadIdx.x; d < L.nDet; d += blockDim.x) {
    float sum = 0.f;
    for (int i = 0; i < nS; i++) {
      const int t = (GEOM == kParallel) ? d : d * nS + i;
      float rx, ry, invr = 1.f, cj = 1.f, sj = 0.f;
      if (GEOM == kParallel) {
        rx = sdir[i].x;
        ry = sdir[i].y;
      } else if (GEOM == kEquilinear) {
        rx = fmaf((float)t, stx, rsx);
        ry = fmaf((float)t, sty, rsy);
        invr = rsqrtf(fmaf(rx, rx, ry * ry));
        rx *= invr;
        ry *= invr;
      } else {
        float half = (float)t * hdelta;    // phi_t / 2, phi_t = t * delta
        sincosf(half, &sj, &cj);
        float cphi = fmaf(-2.f * sj, sj, 1.f), sphi = 2.f * sj * cj;
        float dxv = CD * (fca0 * cphi - fsa0 * sphi), dyv = CD * (fsa0 * cphi + fca0 * sphi);
        rx = dxv - Sx;
        ry = dyv - Sy;
        invr = rsqrtf(fmaf(rx, rx, ry * ry));
        rx *= invr;
        ry *= invr;
      }
      for (int k = 0; k < nElem; k++) {
        const ElemView& e = ev[k * nSub + (GEOM == kParallel ? i : 0)];
        if (!e.live) continue;
        float rho;
        if (GEOM == kEquiangular) {
          float x = ((float)(e.tcI - t) + e.tcF) * hdelta;
          float cf = fmaf(e.cpsi, cj, e.spsi * sj);
          rho = e.kB * cf * sin_series(x) * invr;
        } else {
          float dt = (float)(t - e.tcI) - e.tcF;
          rho = e.kB * dt * invr;
        }
        // cull against the outline box's circumcircle
        float rhob = rho + (rx * e.dcby - ry * e.dcbx);
        const float arhob = fabsf(rhob);
        if (arhob > e.rbox) continue;
        float ra, rb;
        if (GEOM == kParallel) { ra = e.ra; rb = e.rb; }
        else { ra = rx * e.ca + ry * e.sa; rb = -rx * e.sa + ry * e.ca; }
        float ch = element_chord(e, rho, ra, rb);
        if (ch <= 0.f) continue;
        int bt = arhob < e.rin ? 1 : box_test(e, rho, rx, ry);
        if (bt == 0) {
          // repeat the reference's FP64 box clip on this ray's end points
          const PElem& pe = elems[k];
          double lim[4] = {pe.bx0, pe.by0, pe.bx1, pe.by1};
          double xd, yd, xs, ys;
          if (GEOM == kEquiangular) {
            double a = g.alpha0 + (double)t * g.delta;
            double sa, ca;
            sincos(a, &sa, &ca);
            xd = L.centerDetectorLength * ca;
            yd = L.centerDetectorLength * sa;
            xs = g.S0x;
            ys = g.S0y;
          } else {
            xs = g.S0x + (GEOM == kParallel ? d * g.dSx : 0.0);
            ys = g.S0y + (GEOM == kParallel ? d * g.dSy : 0.0);
            int tt = d * nS + i;
            xd = g.D0x + (double)tt * g.dDx;
            yd = g.D0y + (double)tt * g.dDy;
          }
          bt = clip_rect_fp64(xd, yd, xs, ys, lim) ? 1 : -1;
        }
        if (bt < 0) continue;
        sum = fmaf(ch, e.atten, sum);
      }
    }
    sino[(size_t)(L.rowOffset + view) * L.pitch + d] = sum / (float)nS;
  }
}

__global__ void unit_pulse_kernel(float* sino, int nViews, int nDet, int pitch, int rowOffset) {
  int v = blockIdx.x;
  for (int d = threadIdx.x; d < nDet; d += blockDim.x)
    sino[(size_t)(rowOffset + v) * pitch + d] = (d == nDet / 2) ? 1.f : 0.f;
}

cudaError_t launch_raysum(const RaysumLaunch& L, cudaStream_t s) {
  if (L.nViews <= 0) return cudaSuccess;
  int nSub = (L.geometry == kParallel) ? L.nSample : 1;
  size_t smem = dir_table_offset((L.nElem > 0 ? L.nElem : 1) * nSub) +
                sizeof(float2) * (size_t)L.nSample;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  const int nSlices = L.nSlices > 0 ? L.nSlices : 1;
  if (nSlices > 65535) return cudaErrorInvalidConfiguration;
  dim3 grid(L.nViews, nSlices), block(128);
  switch (L.geometry) {
    case kParallel:
      if (smem > 48 * 1024)
        cudaFuncSetAttribute(raysum_kernel<kParallel>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      raysum_kernel<kParallel><<<grid, block, smem, s>>>(L);
      break;
    case kEquilinear:
      if (smem > 48 * 1024)
        cudaFuncSetAttribute(raysum_kernel<kEquilinear>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      raysum_kernel<kEquilinear><<<grid, block, smem, s>>>(L);
      break;
    default:
      if (smem > 48 * 1024)
        cudaFuncSetAttribute(raysum_kernel<kEquiangular>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      raysum_kernel<kEquiangular><<<grid, block, smem, s>>>(L);
      break;
  }
  return cudaGetLastError();
}

cudaError_t launch_unit_pulse(float* sino, int nViews, int nDet, int pitch, int rowOffset,
                              cudaStream_t s) {
  if (nViews <= 0) return cudaSuccess;
  unit_pulse_kernel<<<nViews, 128, 0, s>>>(sino, nViews, nDet, pitch, rowOffset);
  return cudaGetLastError();
}

}  // namespace ctgpu
