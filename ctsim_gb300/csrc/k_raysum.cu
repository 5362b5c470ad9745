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
// margin of the box boundary are decided in FP64 on their end points (the
// line-box test that the reference's Cohen-Sutherland clip amounts to here).
//
// One CTA per view: the per-view FP64 setup is paid once per view.
#include <algorithm>
#include <array>
#include <cmath>

#include "ctgpu_internal.h"
#include "k_fp64.cuh"

namespace ctgpu {

namespace {

struct ElemView {
  // in the order the ray loop reads them, as 16-byte words:
  // [0] rays t outside [tlo, thi] cannot reach the outline box's circumcircle
  // (tlo > thi: no ray of this view meets the element); t_c = tcI + tcF with
  // ftc = (float)tcI
  int tlo, thi;
  float ftc, tcF;
  // [16] rho = kB * (t - t_c) (times 1/|r| for fan beams); equiangular:
  // cos/sin of psi'; circumscribed radius of the outline box
  float kB, cpsi, spsi, rbox;
  // [32] outline box centre minus element centre, its inscribed radius less
  // the margin, element type
  float dcbx, dcby, rin;
  int type;
  // [48] E = (ra/u)^2 + (rb/v)^2 of a unit ray direction (rx, ry) as a
  // quadratic form, E = qa rx^2 + qb rx ry + qc ry^2, and u v (ellipse chords)
  float qa, qb, qc, uv;
  // [64] outline box half sizes, attenuation
  float hx, hy, atten;
  int tcI;
  // [80] element rotation and half sizes (other element types)
  float ca, sa, u, v;
  // [96] parallel: ray direction in the element frame
  float ra, rb;
  int pad0, pad1;
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

// sqrt(x) for x >= 0 from the hardware reciprocal square root (a few ulp)
__device__ __forceinline__ float sqrt_fast(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }

// Chord of the line with unit direction (rx, ry) (world frame; (ra, rb) in the
// element frame) at signed distance rho from the element centre.  Ellipse:
// with E = (ra/u)^2 + (rb/v)^2 the half-chord reaches h = u v sqrt(E), and the
// chord is 2 sqrt(h^2 - rho^2) / (E u v) (factored as (h - |rho|)(h + |rho|)).
__device__ float element_chord(const ElemView& e, float rho, float rx, float ry, float ra,
                               float rb) {
  float u = e.u, v = e.v;
  if (e.type == kEllipse) {
    const float E = fmaf(rx * rx, e.qa, fmaf(rx * ry, e.qb, ry * ry * e.qc));
    const float h = e.uv * sqrt_fast(E);
    const float as = fabsf(rho);
    if (as >= h) return 0.f;
    const float hc = sqrt_fast((h - as) * (h + as));
    return __fdividef(2.f * hc, E * e.uv);
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

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// element_chord's ellipse case from the record's [48] word (qa, qb, qc, uv)
__device__ __forceinline__ float ellipse_chord(float4 q, float rho, float rx, float ry) {
  const float E = fmaf(rx * rx, q.x, fmaf(rx * ry, q.y, ry * ry * q.z));
  const float h = q.w * sqrt_fast(E);
  const float as = fabsf(rho);
  if (as >= h) return 0.f;
  const float hc = sqrt_fast((h - as) * (h + as));
  return __fdividef(2.f * hc, E * q.w);
}

// Does the line through the ray's end points S and D meet the outline box
// [bx0, bx1] x [by0, by1] (FP64)?  The box's centre C lies within its
// half-width along the line's normal: |cross(D - S, C - S)| <= hx |dy| + hy |dx|
// (both sides times |D - S|, so no square root or division).  The reference's
// Cohen-Sutherland clip of the segment S-D (libctsupport/clip.cpp:331-395)
// keeps exactly the segments whose line does this: both end points lie
// outside the view circle that holds the box.
__device__ __forceinline__ bool line_meets_box_fp64(double xs, double ys, double xd, double yd,
                                                    const PElem& pe) {
  const double dx = xd - xs, dy = yd - ys;
  const double hx = 0.5 * (pe.bx1 - pe.bx0), hy = 0.5 * (pe.by1 - pe.by0);
  const double cx = 0.5 * (pe.bx0 + pe.bx1) - xs, cy = 0.5 * (pe.by0 + pe.by1) - ys;
  return fabs(dx * cy - dy * cx) <= hx * fabs(dy) + hy * fabs(dx);
}

// FP32 test of the infinite ray line against the element's outline box:
// +1 clearly hits, -1 clearly misses, 0 within the rounding margin.  The line
// at distance |rhob| from the box centre meets the box exactly when
// |rhob| <= hx |ry| + hy |rx| (the box's half-width along the line's normal).
__device__ __forceinline__ int box_test(float hx, float hy, float rhob, float rx, float ry) {
  const float m = fmaf(hx, fabsf(ry), hy * fabsf(rx)) - fabsf(rhob);
  const float margin = 1e-5f * (hx + hy) + 1e-9f;
  if (m > margin) return 1;
  if (m < -margin) return -1;
  return 0;
}

__device__ __forceinline__ void split_root(double t, int& ti, float& tf) {
  double fl = floor(t);
  if (fl > 2.0e9) fl = 2.0e9;
  if (fl < -2.0e9) fl = -2.0e9;
  ti = (int)fl;
  tf = (float)(t - fl);
}

// Ray indices whose lines can meet the element: an early-out ahead of the
// rays' exact test, so it only has to contain them -- tangents from the
// source, widened by two rays.  An ellipse's rays are those that meet the
// ellipse itself (a ray with a chord does); other elements' those within the
// outline box's circumcircle (centre B, radius rbox).  Parallel rays:
// |rho_B(d)| = |A - d B| <= R is an interval.  Fan rays: the two tangents from
// the source, mapped to ray indices (detector line or arc).  The radius is
// widened well past the FP32 rounding of the rays' own tests.
template <int GEOM>
__device__ void ray_range(const RaysumLaunch& L, const RayView& g, const PElem& pe, int sub,
                          ElemView& e) {
  const int kAll = 1 << 30;
  e.tlo = -kAll;
  e.thi = kAll;
  const bool ell = pe.type == kEllipse;
  if (GEOM == kParallel) {
    double rx = (g.D0x + sub * g.dDx) - g.S0x, ry = (g.D0y + sub * g.dDy) - g.S0y;
    const double inv = rsqrt_nr(rx * rx + ry * ry);
    rx *= inv;
    ry *= inv;
    // the lines within R of the point B: an ellipse's own centre and its
    // half-width across the rays, sqrt(u^2 (n.a1)^2 + v^2 (n.a2)^2) for the
    // rays' normal n and the element axes a1, a2; other elements the outline
    // box's circumcircle
    double Bx, By, R;
    if (ell) {
      const double na1 = rx * pe.sinr - ry * pe.cosr, na2 = rx * pe.cosr + ry * pe.sinr;
      const double h2 = pe.u * pe.u * na1 * na1 + pe.v * pe.v * na2 * na2;
      Bx = pe.cx;
      By = pe.cy;
      R = 1.0001 * (h2 * rsqrt_nr(h2)) + 1e-6;
    } else {
      Bx = pe.cx + (double)pe.dcbx;
      By = pe.cy + (double)pe.dcby;
      R = 1.0001 * (double)pe.rbox + 1e-4 * (fabs(pe.dcbx) + fabs(pe.dcby)) + 1e-30;
    }
    const double A = cross2(rx, ry, Bx - g.S0x, By - g.S0y), B = cross2(rx, ry, g.dSx, g.dSy);
    if (B == 0.0) return;
    const double iB = rcp_nr(B), t1 = (A - R) * iB, t2 = (A + R) * iB;
    const double pad = 2.0 + 1e-5 * (fabs(t1) + fabs(t2));
    double lo = fmin(t1, t2) - pad, hi = fmax(t1, t2) + pad;
    if (!(lo == lo) || !(hi == hi)) return;
    lo = fmax(lo, -(double)kAll);
    hi = fmin(hi, (double)kAll);
    e.tlo = (int)floor(lo);
    e.thi = (int)ceil(hi);
  } else {
    // fan beams in FP32 (the bounds only have to contain the rays): the two
    // tangents from the source
    float ux[2], uy[2];
    if (ell) {
      // to the ellipse itself: in the element frame scaled to the unit circle
      // the source sits at p, the tangent points at angle(p) +- acos(1/|p|)
      const float ct = (float)pe.cosr, st = (float)pe.sinr, eu = (float)pe.u, ev = (float)pe.v;
      const float dxs = (float)(g.S0x - pe.cx), dys = (float)(g.S0y - pe.cy);
      const float px = (ct * dxs + st * dys) / eu, py = (ct * dys - st * dxs) / ev;
      const float pn2 = px * px + py * py;
      if (!(pn2 > 1.0201f)) return;   // the source within 1.01 of the ellipse's size
      const float ip = rsqrtf(pn2);
      const float ca = ip, sa = sqrtf(fmaxf(0.f, 1.f - ip * ip));
      const float qx = px * ip, qy = py * ip;
      for (int k = 0; k < 2; k++) {
        const float sg = k ? -1.f : 1.f;
        const float tx = qx * ca - sg * qy * sa, ty = qy * ca + sg * qx * sa;
        // tangent point minus source, back in the world frame
        const float ex = ct * eu * tx - st * ev * ty - dxs, ey = st * eu * tx + ct * ev * ty - dys;
        const float il = rsqrtf(ex * ex + ey * ey);
        ux[k] = ex * il;
        uy[k] = ey * il;
      }
    } else {
      // to the outline box's circumcircle
      const float R = 1.0001f * pe.rbox + 1e-4f * (fabsf(pe.dcbx) + fabsf(pe.dcby)) + 1e-30f;
      const float wx = (float)(pe.cx - g.S0x) + pe.dcbx, wy = (float)(pe.cy - g.S0y) + pe.dcby;
      const float dist = sqrtf(wx * wx + wy * wy);
      if (!(dist > 1.01f * R)) return;
      const float sb = R / dist;
      const float cb = sqrtf(1.f - sb * sb);
      ux[0] = (wx * cb - wy * sb) / dist;
      ux[1] = (wx * cb + wy * sb) / dist;
      uy[0] = (wy * cb + wx * sb) / dist;
      uy[1] = (wy * cb - wx * sb) / dist;
    }
    float tt[2];
    if (GEOM == kEquilinear) {
      // both tangents must meet the detector line on the same side
      const float d0 = g.stx * uy[0] - g.sty * ux[0], d1 = g.stx * uy[1] - g.sty * ux[1];
      if ((d0 > 0.f) != (d1 > 0.f)) return;
    }
    for (int k = 0; k < 2; k++) {
      if (GEOM == kEquilinear) {
        const float den = g.stx * uy[k] - g.sty * ux[k];
        if (fabsf(den) < 1e-30f) return;
        tt[k] = -(g.rsx * uy[k] - g.rsy * ux[k]) / den;
      } else {
        // far crossing of the tangent with the detector arc |p| = CD, as a
        // ray index from its angle about the arc's middle
        const float Sx = g.Sx, Sy = g.Sy, CD = (float)L.centerDetectorLength;
        const float su = Sx * ux[k] + Sy * uy[k];
        const float disc = su * su - (Sx * Sx + Sy * Sy - CD * CD);
        if (!(disc >= 0.f)) return;
        const float lam = -su + sqrtf(disc);
        const float Dx = Sx + lam * ux[k], Dy = Sy + lam * uy[k];
        const float cm = g.cmf, sm = g.smf;
        tt[k] = (atan2f(cm * Dy - sm * Dx, cm * Dx + sm * Dy) + g.midRelf) * g.invDeltaf;
      }
    }
    // the FP32 pad also covers the rounding of lo and hi themselves
    const float pad = 2.f + 1e-5f * (fabsf(tt[0]) + fabsf(tt[1]));
    float lo = fminf(tt[0], tt[1]) - pad, hi = fmaxf(tt[0], tt[1]) + pad;
    if (!(lo == lo) || !(hi == hi)) return;
    lo = fmaxf(lo, -(float)kAll);
    hi = fminf(hi, (float)kAll);
    e.tlo = (int)floorf(lo);
    e.thi = (int)ceilf(hi);
  }
}

// FP64 set-up of one (view, element[, ray sample]) record.
template <int GEOM>
__device__ void setup_element(const RaysumLaunch& L, const RayView& g, const float2* sdir,
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
  e.qa = pe.qa;
  e.qb = pe.qb;
  e.qc = pe.qc;
  e.uv = pe.uv;
  e.cpsi = e.spsi = 0.f;
  e.ra = e.rb = 0.f;
  e.kB = 0.f;
  e.tcI = 0;
  e.tcF = 0.f;
  e.ftc = 0.f;
  e.tlo = 1;   // no ray until ray_range below
  e.thi = 0;
  if (pe.type < 0) return;   // absent from this view (3-D phantom cross-section)
  if (GEOM == kParallel) {
    // ray direction of sub-sample `sub` (independent of the detector index)
    double rx = (g.D0x + sub * g.dDx) - g.S0x, ry = (g.D0y + sub * g.dDy) - g.S0y;
    double inv = rsqrt_nr(rx * rx + ry * ry);
    rx *= inv;
    ry *= inv;
    double wx = pe.cx - g.S0x, wy = pe.cy - g.S0y;
    double A = cross2(rx, ry, wx, wy), B = cross2(rx, ry, g.dSx, g.dSy);
    // rho(d) = A - d B
    if (B == 0.0) return;
    split_root(A * rcp_nr(B), e.tcI, e.tcF);
    e.kB = (float)(-B);
    e.ra = (float)(rx * pe.cosr + ry * pe.sinr);
    e.rb = (float)(-rx * pe.sinr + ry * pe.cosr);
  } else if (GEOM == kEquilinear) {
    double wx = pe.cx - g.S0x, wy = pe.cy - g.S0y;
    double A = cross2(g.D0x - g.S0x, g.D0y - g.S0y, wx, wy);
    double B = cross2(g.dDx, g.dDy, wx, wy);
    if (B == 0.0) return;
    split_root(-A * rcp_nr(B), e.tcI, e.tcF);
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
    const double w2 = wx * wx + wy * wy;
    const double iw = rsqrt_nr(w2), wn = w2 * iw;
    const double q = cross2(g.S0x, g.S0y, wx, wy) * iw * L.invCD;
    if (!(fabs(q) <= 1.0)) return;
    const double cb2 = (1.0 - q) * (1.0 + q);
    const double cb = cb2 > 1e-300 ? cb2 * rsqrt_nr(cb2) : sqrt(cb2);
    // of the solutions u1 = ((wx cb + wy q), (wy cb - wx q)) / |w| and
    // u2 = -((wx cb - wy q), (wy cb + wx q)) / |w|, the one nearer the arc's
    // middle, chosen in FP32 (the two are far apart for any element whose rays
    // reach the detector) and built in FP64
    const float wxf = (float)wx, wyf = (float)wy, cbf = (float)cb, qf = (float)q;
    const float d1 = fmaf(wxf, cbf, wyf * qf) * g.cmf + fmaf(wyf, cbf, -wxf * qf) * g.smf;
    const float d2 = -fmaf(wxf, cbf, -wyf * qf) * g.cmf - fmaf(wyf, cbf, wxf * qf) * g.smf;
    const double sg = d1 >= d2 ? 1.0 : -1.0;
    const double ux = sg * (wx * cb + sg * wy * q) * iw, uy = sg * (wy * cb - sg * wx * q) * iw;
    const double rel =
        atan2_tab(g.cm * uy - g.sm * ux, g.cm * ux + g.sm * uy, L.atan64) + g.midRel;
    split_root(rel * g.invDelta, e.tcI, e.tcF);
    e.kB = (float)(2.0 * CD * wn);
    // psi = theta_w - (a + alpha0)/2 = (theta_w - alpha0) - rel/2 enters only
    // through its cosine and sine: FP32
    const float thw0 = atan2f(g.ca0 * wyf - g.sa0 * wxf, g.ca0 * wxf + g.sa0 * wyf);
    float sp, cp;
    sincosf(thw0 - 0.5f * (float)rel, &sp, &cp);
    e.cpsi = cp;
    e.spsi = sp;
  }
  e.ftc = (float)e.tcI;
  ray_range<GEOM>(L, g, pe, sub, e);
}

}  // namespace

// Views view0 .. view0 + nvb - 1 of one phantom's sinogram (ev0: the block's
// shared memory, the views' records one after another, then their parallel
// ray directions).
template <int GEOM>
__device__ __forceinline__ void ray_block(const RaysumLaunch& L, int view0, int nvb, int z,
                                          ElemView* ev0) {
  const int nS = L.nSample;
  const int nSub = (GEOM == kParallel) ? nS : 1;
  const PElem* elems0 = L.elems;
  int off = 0, nElem = L.nElem;
  float* sino = L.sino + (size_t)z * L.sliceStride;
  if (L.elemOffset) {
    off = L.elemOffset[z];
    nElem = L.elemOffset[z + 1] - off;
    elems0 += off;
  }
  const int recStride = L.nElem * nSub;   // shared-memory records per view
  // the views' (element, ray sample) records, built in FP64 by the block's
  // first threads straight into shared memory.  FP64 runs at 1/64 of the FP32
  // rate here and these warps are partly idle, but their set-up overlaps the
  // rays of the SM's other blocks, and one set-up pass serves the rays of
  // several views.  Measured on 64 phantoms x 720 views against a separate
  // full-warp set-up launch: equiangular 0.516 -> 0.510 ms with one view per
  // block, 0.452 ms with 4; equilinear 0.442 -> 0.379 / 0.355 ms; parallel
  // with 3 rays per detector 1.177 -> 0.943 ms, 0.921 ms with 2 views (same
  // sums, bit for bit)
  {
    const int per = nElem * nSub;
    for (int k = threadIdx.x; k < per * nvb; k += blockDim.x) {
      const int j = k / per, kk = k - j * per;
      const PElem* el = elems0 + (L.elemsPerView ? (size_t)(view0 + j) * nElem : 0);
      setup_element<GEOM>(L, L.views[view0 + j], L.sdirs, el[kk / nSub], kk % nSub,
                          ev0[j * recStride + kk]);
    }
  }
  float2* sdir0 = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(ev0) +
                                            dir_table_offset(nvb * recStride));
  if (GEOM == kParallel)
    for (int i = threadIdx.x; i < nS * nvb; i += blockDim.x)
      sdir0[i] = L.sdirs[(size_t)view0 * nS + i];
  __syncthreads();

  for (int j = 0; j < nvb; j++) {
    const int view = view0 + j;
    const PElem* elems = elems0 + (L.elemsPerView ? (size_t)view * nElem : 0);
    const ElemView* ev = ev0 + j * recStride;
    const float2* sdir = sdir0 + j * nS;   // per sub-sample
    const RayView& g = L.views[view];
    const float rsx = g.rsx, rsy = g.rsy, stx = g.stx, sty = g.sty;
    const float hdelta = g.hdelta, fca0 = g.ca0, fsa0 = g.sa0, Sx = g.Sx, Sy = g.Sy;
    const float CD = (float)L.centerDetectorLength;

    // ray indices as floats by float arithmetic (exact below 2^24), not by
    // int-to-float conversions
    const float fnS = (float)nS, fstep = (float)blockDim.x;
    float fd = (float)threadIdx.x;
    for (int d = threadIdx.x; d < L.nDet; d += blockDim.x, fd += fstep) {
      float sum = 0.f;
      float fi = 0.f;
      for (int i = 0; i < nS; i++, fi += 1.f) {
        const int t = (GEOM == kParallel) ? d : d * nS + i;
        const float ft = (GEOM == kParallel) ? fd : fmaf(fd, fnS, fi);
        float rx, ry, invr = 1.f, cj = 1.f, sj = 0.f;
        if (GEOM == kParallel) {
          rx = sdir[i].x;
          ry = sdir[i].y;
        } else if (GEOM == kEquilinear) {
          rx = fmaf(ft, stx, rsx);
          ry = fmaf(ft, sty, rsy);
          invr = rsqrtf(fmaf(rx, rx, ry * ry));
          rx *= invr;
          ry *= invr;
        } else {
          // cos, sin of phi_t / 2 (phi_t = t * delta) from the scanner's table
          const float2 cs = __ldg(&L.arcHalf[t]);
          cj = cs.x;
          sj = cs.y;
          float cphi = fmaf(-2.f * sj, sj, 1.f), sphi = 2.f * sj * cj;
          float dxv = CD * (fca0 * cphi - fsa0 * sphi), dyv = CD * (fsa0 * cphi + fca0 * sphi);
          rx = dxv - Sx;
          ry = dyv - Sy;
          invr = rsqrtf(fmaf(rx, rx, ry * ry));
          rx *= invr;
          ry *= invr;
        }
        // the elements whose ray range meets this warp's rays: lane j tests
        // element kb + j, a ballot collects them, and the loop visits them in
        // ascending order (the sums keep their order).  The warp's lanes in this
        // iteration are the detectors dw0 .. dwm, all of them here.
        const int dw0 = d - (int)(threadIdx.x & 31), dwm = min(dw0 + 31, L.nDet - 1);
        const unsigned wmask = dwm - dw0 >= 31 ? 0xffffffffu : (1u << (dwm - dw0 + 1)) - 1u;
        const int twlo = (GEOM == kParallel) ? dw0 : dw0 * nS + i;
        const int twhi = (GEOM == kParallel) ? dwm : dwm * nS + i;
        for (int kb = 0; kb < nElem; kb += 32) {
          const int kl = kb + (int)(threadIdx.x & 31);
          bool meets = false;
          if (kl < nElem) {
            const int2 r = *reinterpret_cast<const int2*>(&ev[kl * nSub + (GEOM == kParallel ? i : 0)]);
            meets = !(twhi < r.x || twlo > r.y);
          }
          unsigned todo = __ballot_sync(wmask, meets);
          while (todo) {
            const int k = kb + __ffs(todo) - 1;
            todo &= todo - 1;
            const ElemView& e = ev[k * nSub + (GEOM == kParallel ? i : 0)];
            const int4 hdr = *reinterpret_cast<const int4*>(&e);
            if (t < hdr.x || t > hdr.y) continue;
            // integers below 2^24: (float)tcI - ft is the exact (float)(tcI - t)
            const float ftc = __int_as_float(hdr.z), tcF = __int_as_float(hdr.w);
            const float4 w1 = ld4(&e.kB);     // kB, cpsi, spsi, rbox
            float rho;
            if (GEOM == kEquiangular) {
              float x = ((ftc - ft) + tcF) * hdelta;
              float cf = fmaf(w1.y, cj, w1.z * sj);
              rho = w1.x * cf * sin_series(x) * invr;
            } else {
              float dt = (ft - ftc) - tcF;
              rho = w1.x * dt * invr;
            }
            // cull against the outline box's circumcircle
            const float4 w2 = ld4(&e.dcbx);   // dcbx, dcby, rin, type
            float rhob = rho + (rx * w2.y - ry * w2.x);
            const float arhob = fabsf(rhob);
            if (arhob > w1.w) continue;
            float ch;
            if (__float_as_int(w2.w) == kEllipse) {
              ch = ellipse_chord(ld4(&e.qa), rho, rx, ry);
            } else {
              float ra, rb;
              if (GEOM == kParallel) { ra = e.ra; rb = e.rb; }
              else { ra = rx * e.ca + ry * e.sa; rb = -rx * e.sa + ry * e.ca; }
              ch = element_chord(e, rho, rx, ry, ra, rb);
            }
            if (ch <= 0.f) continue;
            const float4 w4 = ld4(&e.hx);     // hx, hy, atten, tcI
            int bt = arhob < w2.z ? 1 : box_test(w4.x, w4.y, rhob, rx, ry);
            if (bt == 0) {
              // within the FP32 test's margin: decide in FP64 on this ray's end
              // points whether its line meets the outline box
              const PElem& pe = elems[k];
              double xd, yd, xs, ys;
              if (GEOM == kEquiangular) {
                // detector point at arc angle alpha0 + t delta, by the angle sum
                const double2 a = L.arc[t];
                xd = L.centerDetectorLength * (g.c0 * a.x - g.s0 * a.y);
                yd = L.centerDetectorLength * (g.s0 * a.x + g.c0 * a.y);
                xs = g.S0x;
                ys = g.S0y;
              } else {
                xs = g.S0x + (GEOM == kParallel ? d * g.dSx : 0.0);
                ys = g.S0y + (GEOM == kParallel ? d * g.dSy : 0.0);
                int tt = d * nS + i;
                xd = g.D0x + (double)tt * g.dDx;
                yd = g.D0y + (double)tt * g.dDy;
              }
              bt = line_meets_box_fp64(xs, ys, xd, yd, pe) ? 1 : -1;
            }
            if (bt < 0) continue;
            sum = fmaf(ch, w4.z, sum);
          }
        }
      }
      sino[(size_t)(L.rowOffset + view) * L.pitch + d] = sum / fnS;
    }
  }
}

template <int GEOM>
__global__ void __launch_bounds__(128) raysum_kernel(RaysumLaunch L) {
  extern __shared__ __align__(16) ElemView ev[];
  const int v0 = blockIdx.x * L.viewsPerBlock;
  ray_block<GEOM>(L, v0, min(L.viewsPerBlock, L.nViews - v0), blockIdx.y, ev);
}

// Many scans in one launch each: problem k's descriptor is probs[k] (in
// device memory), and its blocks are blockStart[k] .. blockStart[k+1) of the
// grid, one per viewsPerBlock views.
__device__ __forceinline__ int problem_of_block(const int* __restrict__ blockStart, int n) {
  int lo = 0, hi = n - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (blockStart[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(128, 4) raysum_multi_kernel(const RaysumLaunch* __restrict__ probs,
                                                           const int* __restrict__ blockStart,
                                                           int n) {
  extern __shared__ __align__(16) ElemView ev[];
  const int k = problem_of_block(blockStart, n);
  const RaysumLaunch& L = probs[k];
  const int v0 = (blockIdx.x - blockStart[k]) * L.viewsPerBlock;
  const int nvb = min(L.viewsPerBlock, L.nViews - v0);
  switch (L.geometry) {
    case kParallel: ray_block<kParallel>(L, v0, nvb, 0, ev); break;
    case kEquilinear: ray_block<kEquilinear>(L, v0, nvb, 0, ev); break;
    default: ray_block<kEquiangular>(L, v0, nvb, 0, ev); break;
  }
}

__global__ void unit_pulse_kernel(float* sino, int nViews, int nDet, int pitch, int rowOffset) {
  int v = blockIdx.x;
  for (int d = threadIdx.x; d < nDet; d += blockDim.x)
    sino[(size_t)(rowOffset + v) * pitch + d] = (d == nDet / 2) ? 1.f : 0.f;
}

template <int GEOM>
static cudaError_t raysum_launch(const RaysumLaunch& L, size_t smem, int nSlices,
                                 cudaStream_t s) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(raysum_kernel<GEOM>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  dim3 grid((L.nViews + L.viewsPerBlock - 1) / L.viewsPerBlock, nSlices);
  raysum_kernel<GEOM><<<grid, 128, smem, s>>>(L);
  return cudaGetLastError();
}

// shared memory of a ray block of vpb views (records, then parallel directions)
static size_t raysum_smem(const RaysumLaunch& L, int vpb) {
  const int nSub = (L.geometry == kParallel) ? L.nSample : 1;
  return dir_table_offset((size_t)vpb * (L.nElem > 0 ? L.nElem : 1) * nSub) +
         sizeof(float2) * (size_t)L.nSample * vpb;
}

// views per ray block: 4, or 2 for several rays per detector (measured best
// of 1, 2, 4, 6, 8 on 64 phantoms x 720 views), fewer where their records
// would not fit the 48 KB a block gets without opting in
static int raysum_views_per_block(const RaysumLaunch& L) {
  const int nSub = (L.geometry == kParallel) ? L.nSample : 1;
  int vpb = nSub > 1 ? 2 : 4;
  while (vpb > 1 && raysum_smem(L, vpb) > 48 * 1024) vpb--;
  return vpb;
}

cudaError_t launch_raysum(const RaysumLaunch& L0, cudaStream_t s) {
  if (L0.nViews <= 0) return cudaSuccess;
  RaysumLaunch L = L0;
  L.invCD = L.centerDetectorLength != 0.0 ? 1.0 / L.centerDetectorLength : 0.0;
  std::copy(atan64_table().v, atan64_table().v + 65, L.atan64);
  L.viewsPerBlock = raysum_views_per_block(L);
  const size_t smem = raysum_smem(L, L.viewsPerBlock);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  const int nSlices = L.nSlices > 0 ? L.nSlices : 1;
  if (nSlices > 65535) return cudaErrorInvalidConfiguration;
  switch (L.geometry) {
    case kParallel: return raysum_launch<kParallel>(L, smem, nSlices, s);
    case kEquilinear: return raysum_launch<kEquilinear>(L, smem, nSlices, s);
    default: return raysum_launch<kEquiangular>(L, smem, nSlices, s);
  }
}

size_t raysum_prepare(RaysumLaunch& L) {
  L.invCD = L.centerDetectorLength != 0.0 ? 1.0 / L.centerDetectorLength : 0.0;
  std::copy(atan64_table().v, atan64_table().v + 65, L.atan64);
  L.viewsPerBlock = raysum_views_per_block(L);
  return raysum_smem(L, L.viewsPerBlock);
}

cudaError_t launch_raysum_multi(const RaysumLaunch* d_probs, const int* d_rayStart,
                                int rayBlocks, int n, size_t smem, cudaStream_t s) {
  if (n <= 0 || rayBlocks <= 0) return cudaSuccess;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(raysum_multi_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  raysum_multi_kernel<<<rayBlocks, 128, smem, s>>>(d_probs, d_rayStart, n);
  return cudaGetLastError();
}

__global__ void ellipsoid_section_kernel(const PElem* base, const double2* zc, int n, int nViews,
                                         double z0, double dz, PElem* out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * nViews) return;
  const int v = idx / n, k = idx % n;
  PElem e = base[k];
  const double d = (z0 + v * dz - zc[k].x) / zc[k].y;
  if (!(fabs(d) < 1.0)) {
    e.type = -1;
  } else {
    const double sc = sqrt((1.0 - d) * (1.0 + d));
    e.u *= sc;
    e.v *= sc;
    e.bx0 = e.cx + sc * (e.bx0 - e.cx);
    e.bx1 = e.cx + sc * (e.bx1 - e.cx);
    e.by0 = e.cy + sc * (e.by0 - e.cy);
    e.by1 = e.cy + sc * (e.by1 - e.cy);
    const double hx = 0.5 * (e.bx1 - e.bx0), hy = 0.5 * (e.by1 - e.by0);
    e.dcbx = (float)(0.5 * (e.bx0 + e.bx1) - e.cx);
    e.dcby = (float)(0.5 * (e.by0 + e.by1) - e.cy);
    e.hx = (float)hx;
    e.hy = (float)hy;
    e.rbox = (float)(sqrt(hx * hx + hy * hy) * (1.0 + 1e-5) + 1e-7);
    e.rin = (float)(fmin(hx, hy) - 2e-5 * (hx + hy) - 1e-7);
    set_elem_quadratic(e);
  }
  out[idx] = e;
}

cudaError_t launch_ellipsoid_sections(const PElem* base, const double2* zc, int n, int nViews,
                                      double z0, double dz, PElem* out, cudaStream_t s) {
  if (n <= 0 || nViews <= 0) return cudaSuccess;
  const long long total = (long long)n * nViews;
  if (total > (1LL << 31) - 256) return cudaErrorInvalidValue;
  ellipsoid_section_kernel<<<(unsigned)((total + 127) / 128), 128, 0, s>>>(base, zc, n, nViews, z0,
                                                                          dz, out);
  return cudaGetLastError();
}

cudaError_t launch_unit_pulse(float* sino, int nViews, int nDet, int pitch, int rowOffset,
                              cudaStream_t s) {
  if (nViews <= 0) return cudaSuccess;
  unit_pulse_kernel<<<nViews, 128, 0, s>>>(sino, nViews, nDet, pitch, rowOffset);
  return cudaGetLastError();
}

}  // namespace ctgpu

// ---------------------------------------------------------------------------
// Gradient of the ray-sums with respect to the ellipses' parameters (no
// reference counterpart).  For a ray with unit direction r through the point
// S, an ellipse with centre W, semi-axes u, v, rotation theta and attenuation
// a has signed distance rho = cross(r, W - S) and, with (ra, rb) = r in the
// ellipse frame, Q = v^2 ra^2 + u^2 rb^2, hc^2 = Q - rho^2, the chord
//   c = 2 u v hc / Q   (hc^2 > 0; 0 otherwise)
// whose partial derivatives are
//   dc/drho = -2 u v rho / (Q hc)              drho/dW = (-ry, rx)
//   dc/dQ   = u v (2 rho^2 - Q) / (hc Q^2)     dQ/du = 2 u rb^2, dQ/dv = 2 v ra^2,
//   dc/du  |= 2 v hc / Q,  dc/dv |= 2 u hc / Q  dQ/dtheta = 2 ra rb (v^2 - u^2)
// A ray counts for an ellipse as in the forward model: hc^2 > 0 and accepted
// by the reference's outline-box clip (held fixed in the derivative).  The
// derivative grows like 1/hc at tangency, so the terms are formed in FP64
// (FP32's rounding of hc^2 would dominate there); the detector value is the
// mean over its ray samples.  One CTA per view: the rays are staged in
// shared memory, then per ellipse each thread accumulates its rays' six
// terms, warps reduce, and the CTA's totals go to FP64 global accumulators.
// ---------------------------------------------------------------------------
namespace ctgpu {

struct GradRay { double rx, ry, sx, sy, xd, yd, g; };

template <int GEOM>
__global__ void __launch_bounds__(128) raysum_ellipse_grad_kernel(RaysumLaunch L,
                                                                  const float* __restrict__ gsino,
                                                                  double* __restrict__ grad) {
  extern __shared__ __align__(16) unsigned char smg[];
  GradRay* rays = reinterpret_cast<GradRay*>(smg);
  const int view = blockIdx.x;
  const RayView& g = L.views[view];
  const int nS = L.nSample, nRay = L.nDet * nS;
  const float* gv = gsino + (size_t)(L.rowOffset + view) * L.pitch;
  for (int t = threadIdx.x; t < nRay; t += blockDim.x) {
    const int d = t / nS;
    GradRay R;
    double sx = g.S0x, sy = g.S0y, px, py;
    if (GEOM == kEquiangular) {
      double sa, ca;
      sincos(g.alpha0 + (double)t * g.delta, &sa, &ca);
      px = L.centerDetectorLength * ca;
      py = L.centerDetectorLength * sa;
    } else {
      if (GEOM == kParallel) {
        sx += d * g.dSx;
        sy += d * g.dSy;
      }
      px = g.D0x + (double)t * g.dDx;
      py = g.D0y + (double)t * g.dDy;
    }
    double dx = px - sx, dy = py - sy;
    const double n = 1.0 / sqrt(dx * dx + dy * dy);
    R.rx = dx * n;
    R.ry = dy * n;
    R.sx = sx;
    R.sy = sy;
    R.xd = px;
    R.yd = py;
    R.g = (double)gv[d] / nS;
    rays[t] = R;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int k = 0; k < L.nElem; k++) {
    const PElem& pe = L.elems[k];
    const double cx = pe.cx, cy = pe.cy, u = pe.u, v = pe.v;
    const double ct = pe.cosr, st = pe.sinr, at = pe.atten;
    const double bcx = 0.5 * (pe.bx0 + pe.bx1), bcy = 0.5 * (pe.by0 + pe.by1);
    const double rin = fmin(pe.bx1 - pe.bx0, pe.by1 - pe.by0) * 0.5 * (1.0 - 1e-9);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int t = threadIdx.x; t < nRay; t += blockDim.x) {
      const GradRay R = rays[t];
      const double rho = R.rx * (cy - R.sy) - R.ry * (cx - R.sx);
      const double ra = R.rx * ct + R.ry * st, rb = -R.rx * st + R.ry * ct;
      const double Q = v * v * ra * ra + u * u * rb * rb;
      const double h2 = Q - rho * rho;
      if (!(h2 > 0.0)) continue;
      // the forward model's outline-box acceptance: certain inside the box's
      // inscribed circle, else the FP64 line-box test on the ray's end points
      const double rbox = R.rx * (bcy - R.sy) - R.ry * (bcx - R.sx);
      if (!(fabs(rbox) < rin) && !line_meets_box_fp64(R.sx, R.sy, R.xd, R.yd, pe)) continue;
      const double hc = sqrt(h2);
      const double iQ = 1.0 / Q;
      const double c = 2.0 * u * v * hc * iQ;
      const double dcdrho = -2.0 * u * v * rho * iQ / hc;
      const double dcdQ = u * v * (2.0 * rho * rho - Q) * iQ * iQ / hc;
      const double ga = R.g * at;
      acc[0] += ga * dcdrho * -R.ry;                                   // cx
      acc[1] += ga * dcdrho * R.rx;                                    // cy
      acc[2] += ga * (2.0 * v * hc * iQ + dcdQ * 2.0 * u * rb * rb);   // u
      acc[3] += ga * (2.0 * u * hc * iQ + dcdQ * 2.0 * v * ra * ra);   // v
      acc[4] += ga * dcdQ * 2.0 * ra * rb * (v * v - u * u);           // theta (radians)
      acc[5] += R.g * c;                                               // attenuation
    }
#pragma unroll
    for (int j = 0; j < 6; j++) {
      double a = acc[j];
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0) atomicAdd(&grad[6 * k + j], a);
    }
  }
}

cudaError_t launch_raysum_ellipse_grad(const RaysumLaunch& L, const float* gsino, double* grad,
                                       cudaStream_t s) {
  if (L.nViews <= 0 || L.nElem <= 0) return cudaSuccess;
  const size_t smem = sizeof(GradRay) * (size_t)L.nDet * L.nSample;
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  switch (L.geometry) {
    case kParallel:
      if (smem > 48 * 1024)
        cudaFuncSetAttribute(raysum_ellipse_grad_kernel<kParallel>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      raysum_ellipse_grad_kernel<kParallel><<<L.nViews, 128, smem, s>>>(L, gsino, grad);
      break;
    case kEquilinear:
      if (smem > 48 * 1024)
        cudaFuncSetAttribute(raysum_ellipse_grad_kernel<kEquilinear>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      raysum_ellipse_grad_kernel<kEquilinear><<<L.nViews, 128, smem, s>>>(L, gsino, grad);
      break;
    default:
      if (smem > 48 * 1024)
        cudaFuncSetAttribute(raysum_ellipse_grad_kernel<kEquiangular>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      raysum_ellipse_grad_kernel<kEquiangular><<<L.nViews, 128, smem, s>>>(L, gsino, grad);
      break;
  }
  return cudaGetLastError();
}

}  // namespace ctgpu

// ---------------------------------------------------------------------------
// Phantom::convertToImagefile (libctsim/phantom.cpp:462-542), what phm2if does:
// each pixel is the mean over nsample x nsample points of the summed
// attenuation of the elements containing the point
// (PhantomElement::isPointInside, phantom.cpp:913-976).  One thread per pixel;
// the point coordinates are accumulated by the reference's own sequential
// additions (column and row starts from the host), every test is its FP64
// affine map, and the FP32 pixel is updated once per element in list order
// with the reference's FP32-image roundings.
// ---------------------------------------------------------------------------
namespace ctgpu {

__device__ __forceinline__ bool raster_inside(const RasterElem& e, double x, double y) {
  const double xo = x * e.m[0][0] + y * e.m[1][0] + e.m[2][0];
  const double yo = x * e.m[0][1] + y * e.m[1][1] + e.m[2][1];
  double xs = xo, ys = yo;
  switch (e.type) {
    case kRect: return !(xo > 1. || xo < -1. || yo > 1. || yo < -1.);
    case kTriangle: return !(yo < 0. || yo > 1. - xo || yo > 1. + xo);
    case kEllipse:
      if (xo > 1. || xo < -1. || yo > 1. || yo < -1.) return false;
      return !(xo * xo + yo * yo > 1.);
    case kSegment:
      if (xo > 1. || xo < -1. || yo > 0.) return false;
      xs *= e.u;
      ys *= e.v;
      return !(xs * xs + (ys - e.v) * (ys - e.v) > e.u * e.u + e.v * e.v);
    case kSector:
      if (xo > 1. || xo < -1. || yo > 1.) return false;
      if (yo > 1. - xo || yo > 1. + xo) return false;
      xs *= e.u;
      ys *= e.v;
      return !(xs * xs + (ys - e.v) * (ys - e.v) > e.u * e.u + e.v * e.v);
    default: return false;
  }
}

__global__ void raster_kernel(RasterLaunch L) {
  const int ix = blockIdx.x;
  const double x = L.xcol[ix];
  for (int iy = threadIdx.x; iy < L.ny; iy += blockDim.x) {
    const double y = L.yrow[iy];
    float pix = 0.f;
    for (int k = 0; k < L.nElem; k++) {
      const RasterElem& e = L.elems[k];
      double a = 0;
      double xi = x + L.kxofs;
      for (int kx = 0; kx < L.nsample; kx++, xi += L.kxinc) {
        double yi = y + L.kyofs;
        for (int ky = 0; ky < L.nsample; ky++, yi += L.kyinc)
          if (raster_inside(e, xi, yi)) a += e.atten;
      }
      pix = (float)((double)pix + a);
    }
    if (L.nsample > 1) pix = (float)((double)pix * L.factor);
    L.image[(size_t)ix * L.ny + iy] = pix;
  }
}

cudaError_t launch_raster(const RasterLaunch& L, cudaStream_t s) {
  if (L.nx <= 0 || L.ny <= 0) return cudaSuccess;
  raster_kernel<<<L.nx, 128, 0, s>>>(L);
  return cudaGetLastError();
}

}  // namespace ctgpu
