/* ctoracle.c -- TEST INFRASTRUCTURE ONLY (see ctoracle.h).
 *
 * FP64 CPU restatement of the CTSim 5.2.0 simulate -> filter -> backproject path.
 * It follows the reference's algorithms step by step (same loop order, same
 * incremental accumulations, same clipping steps) so that, compiled without
 * floating-point contraction, it reproduces the reference's FP64 arithmetic;
 * tests/golden/ pins it against the reference built from source.  Loops over
 * independent views / image columns are spread over OpenMP threads; the
 * arithmetic per output element does not depend on the thread count.
 *
 * All file:line citations are into CTSim 5.2.0.
 */
#include "ctoracle.h"
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* include/ctsupport.h:167-179 */
#define O_PI      3.14159265358979323846
#define O_HALFPI  1.57079632679489661923
#define O_TWOPI   6.28318530717958647692
#define O_SQRT2   1.414213562373095049
#define O_FEPS    1.0E-6
#define O_DEPS    1.0E-10

typedef double mtx2[3][3];

/* ------------------------------------------------------------------------- */
/* 2-D row-vector affine matrices: libctsupport/xform.cpp:87-148            */
/* ------------------------------------------------------------------------- */
static void m_ident(mtx2 m) {
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) m[r][c] = (r == c) ? 1.0 : 0.0;
}
static void m_xlat(mtx2 m, double x, double y) { m_ident(m); m[2][0] = x; m[2][1] = y; }
static void m_scale(mtx2 m, double sx, double sy) { m_ident(m); m[0][0] = sx; m[1][1] = sy; }
static void m_rot(mtx2 m, double t) {
  double c = cos(t), s = sin(t);
  m_ident(m);
  m[0][0] = c; m[0][1] = s;
  m[1][0] = -s; m[1][1] = c;
}
/* result = a * b (xform.cpp:123-138) */
static void m_mul(mtx2 a, mtx2 b, mtx2 res) {
  mtx2 t;
  for (int r = 0; r < 3; r++)
    for (int c = 0; c < 3; c++) {
      t[r][c] = 0;
      for (int k = 0; k < 3; k++) t[r][c] += a[r][k] * b[k][c];
    }
  memcpy(res, t, sizeof(mtx2));
}
static void m_apply(const double m[3][3], double* x, double* y) {
  double xt = *x * m[0][0] + *y * m[1][0] + m[2][0];
  double yt = *x * m[0][1] + *y * m[1][1] + m[2][1];
  *x = xt; *y = yt;
}

/* libctsupport/mathfuncs.cpp:73-83 */
static double norm_angle(double t) {
  while (t < 0.) t += O_TWOPI;
  while (t >= O_TWOPI) t -= O_TWOPI;
  return t;
}

/* include/ctsupport.h:193 (round half away from zero) */
static long nearest_long(double x) { return x > 0 ? (long)(x + 0.5) : (long)(x - 0.5); }
static int nearest_int(double x) { return x > 0 ? (int)(x + 0.5) : (int)(x - 0.5); }

/* ------------------------------------------------------------------------- */
/* Line clipping: libctsupport/clip.cpp                                     */
/* ------------------------------------------------------------------------- */
/* rectangle region code: clip.cpp:381-395 */
static int rect_code(double x, double y, const double r[4]) {
  int c = 0;
  if (x < r[0]) c = 1;
  else if (x > r[2]) c = 2;
  if (y < r[1]) c += 4;
  else if (y > r[3]) c += 8;
  return c;
}
/* Cohen-Sutherland against [xmin,ymin,xmax,ymax]: clip.cpp:331-366 */
static int clip_rect(double* x1, double* y1, double* x2, double* y2, const double r[4]) {
  int c1 = rect_code(*x1, *y1, r), c2 = rect_code(*x2, *y2, r);
  double x = 0, y = 0;
  while (c1 || c2) {
    if (c1 & c2) return 0;
    int c = c1 ? c1 : c2;
    if (c & 1) { y = *y1 + (*y2 - *y1) * (r[0] - *x1) / (*x2 - *x1); x = r[0]; }
    else if (c & 2) { y = *y1 + (*y2 - *y1) * (r[2] - *x1) / (*x2 - *x1); x = r[2]; }
    else if (c & 4) { x = *x1 + (*x2 - *x1) * (r[1] - *y1) / (*y2 - *y1); y = r[1]; }
    else if (c & 8) { x = *x1 + (*x2 - *x1) * (r[3] - *y1) / (*y2 - *y1); y = r[3]; }
    if (c == c1) { *x1 = x; *y1 = y; c1 = rect_code(*x1, *y1, r); }
    else { *x2 = x; *y2 = y; c2 = rect_code(*x2, *y2, r); }
  }
  return 1;
}
/* circle clip with start/stop angles (both 0 for a full circle): clip.cpp:125-198 */
static int clip_circle(double* x1, double* y1, double* x2, double* y2, double cx, double cy,
                       double radius, double t1, double t2) {
  double xc1 = *x1, yc1 = *y1, xc2 = *x2, yc2 = *y2, ccx = cx, ccy = cy;
  double xtrans = -xc1, ytrans = -yc1;
  xc1 += xtrans; yc1 += ytrans; xc2 += xtrans; yc2 += ytrans; ccx += xtrans; ccy += ytrans;
  double theta = -atan2(yc2, xc2);
  mtx2 rm;
  m_rot(rm, theta);
  m_apply((const double(*)[3])rm, &xc2, &yc2);
  m_apply((const double(*)[3])rm, &ccx, &ccy);
  t1 += theta; t2 += theta;
  t1 = norm_angle(t1); t2 = norm_angle(t2);
  if (xc2 < -O_DEPS || fabs(yc2) > O_FEPS) return 0;
  if (fabs(ccy) > radius) return 0;
  double temp = sqrt(radius * radius - ccy * ccy);
  double xcmin = ccx - temp, xcmax = ccx + temp;
  if (fabs(t2 - t1) < O_DEPS) {
    if (xc1 < xcmin) xc1 = xcmin;
    if (xc2 > xcmax) xc2 = xcmax;
  } else if (t1 < t2) {
    if (t1 < O_PI && t2 > O_PI)
      if (xc1 < xcmin) xc1 = xcmin;
  } else if (t1 > t2) {
    if (t1 < O_PI)
      if (xc1 < xcmin) xc1 = xcmin;
    if (xc2 > xcmax) xc2 = xcmax;
  }
  m_rot(rm, -theta);
  m_apply((const double(*)[3])rm, &xc1, &yc1);
  m_apply((const double(*)[3])rm, &xc2, &yc2);
  xc1 += -xtrans; yc1 += -ytrans; xc2 += -xtrans; yc2 += -ytrans;
  *x1 = xc1; *y1 = yc1; *x2 = xc2; *y2 = yc2;
  return 1;
}
/* triangle region code: clip.cpp:302-316 */
static int tri_code(double x, double y, double m, double b, int clipx) {
  int c = 0;
  if (clipx && y < 0.) c = 1;
  if (y > -m * x + b + O_DEPS) c += 2;
  if (y > m * x + b + O_DEPS) c += 4;
  return c;
}
/* triangle (-u,0),(u,0),(0,v): clip.cpp:242-298 */
static int clip_triangle(double* x1, double* y1, double* x2, double* y2, double u, double v,
                         int clipx) {
  double m = v / u, b = v;
  int c1 = tri_code(*x1, *y1, m, b, clipx), c2 = tri_code(*x2, *y2, m, b, clipx);
  while (c1 || c2) {
    if (c1 & c2) return 0;
    int c = c1 ? c1 : c2;
    double x = 0, y = 0;
    if (c & 1) {
      x = *x1 + (*x2 - *x1) * (0.0 - *y1) / (*y2 - *y1);
      y = 0.0;
    } else if (c & 2) {
      double dx = *x2 - *x1, dy = *y2 - *y1;
      if (fabs(dx) > O_DEPS) x = (-*y1 + b + *x1 * dy / dx) / (m + dy / dx);
      else x = *x1;
      y = -m * x + b;
    } else if (c & 4) {
      double dx = *x2 - *x1, dy = *y2 - *y1;
      if (fabs(dx) > O_DEPS) { x = (*y1 - b - *x1 * dy / dx); x /= (m - dy / dx); }
      else x = *x1;
      y = m * x + b;
    }
    if (c == c1) { *x1 = x; *y1 = y; c1 = tri_code(*x1, *y1, m, b, clipx); }
    else { *x2 = x; *y2 = y; c2 = tri_code(*x2, *y2, m, b, clipx); }
  }
  return 1;
}
/* circular segment below the x-axis: clip.cpp:43-77 */
static int clip_segment(double* x1, double* y1, double* x2, double* y2, double u, double v) {
  double xc1 = *x1 * u, yc1 = *y1 * v, xc2 = *x2 * u, yc2 = *y2 * v;
  if (yc1 > 0. && yc2 > 0.) return 0;
  double radius = sqrt(u * u + v * v);
  if (!clip_circle(&xc1, &yc1, &xc2, &yc2, 0.0, v, radius, 0.0, 0.0)) return 0;
  if (yc1 > 0. && yc2 > 0.) return 0;
  if (yc1 > 0.) {
    xc1 = xc1 + (xc2 - xc1) * (0.0 - yc1) / (yc2 - yc1);
    yc1 = 0.0;
  } else if (yc2 > 0.) {
    xc2 = xc1 + (xc2 - xc1) * (0.0 - yc1) / (yc2 - yc1);
    yc2 = 0.0;
  }
  *x1 = xc1 / u; *y1 = yc1 / v; *x2 = xc2 / u; *y2 = yc2 / v;
  return 1;
}
/* circular sector: clip.cpp:89-111 */
static int clip_sector(double* x1, double* y1, double* x2, double* y2, double u, double v) {
  double xc1 = *x1 * u, yc1 = *y1 * v, xc2 = *x2 * u, yc2 = *y2 * v;
  double radius = sqrt(u * u + v * v);
  if (!clip_circle(&xc1, &yc1, &xc2, &yc2, 0.0, v, radius, 0.0, 0.0)) return 0;
  if (!clip_triangle(&xc1, &yc1, &xc2, &yc2, u, v, 0)) return 0;
  *x1 = xc1 / u; *y1 = yc1 / v; *x2 = xc2 / u; *y2 = yc2 / v;
  return 1;
}

/* ------------------------------------------------------------------------- */
/* Phantom elements: libctsim/phantom.cpp                                   */
/* ------------------------------------------------------------------------- */
int ora_name_to_pelem_type(const char* n) {   /* phantom.cpp:590-607 */
  if (!strcasecmp(n, "rectangle")) return ORA_PELEM_RECTANGLE;
  if (!strcasecmp(n, "triangle")) return ORA_PELEM_TRIANGLE;
  if (!strcasecmp(n, "ellipse")) return ORA_PELEM_ELLIPSE;
  if (!strcasecmp(n, "sector")) return ORA_PELEM_SECTOR;
  if (!strcasecmp(n, "segment")) return ORA_PELEM_SEGMENT;
  return ORA_PELEM_INVALID;
}

/* points per arc: phantom.cpp:821-827 */
static int circle_points(double theta) {
  if (theta <= 0.) theta = 0.;
  if (theta >= O_TWOPI) theta = O_TWOPI;
  return (int)(360 * theta / O_TWOPI + 1.5);
}
/* incremental arc: phantom.cpp:771-793 */
static void arc_points(double* x, double* y, int pts, double xc, double yc, double r,
                       double start, double stop) {
  double th = (stop - start) / (pts - 1);
  double c = cos(th), s = sin(th);
  x[0] = r * cos(start) + xc;
  y[0] = r * sin(start) + yc;
  double xp = x[0] - xc, yp = y[0] - yc;
  for (int i = 1; i < pts; i++) {
    double xn = c * xp - s * yp, yn = s * xp + c * yp;
    x[i] = xn + xc; y[i] = yn + yc;
    xp = xn; yp = yn;
  }
}

/* PhantomElement ctor: transforms (phantom.cpp:629-655) and outline bbox (:669-756) */
static void pelem_setup(ora_pelem* e) {
  mtx2 t;
  m_scale(e->obj2phm, e->u, e->v);
  m_rot(t, e->rot); m_mul(e->obj2phm, t, e->obj2phm);
  m_xlat(t, e->cx, e->cy); m_mul(e->obj2phm, t, e->obj2phm);
  m_xlat(e->phm2obj, -e->cx, -e->cy);
  m_rot(t, -e->rot); m_mul(e->phm2obj, t, e->phm2obj);
  m_scale(t, 1 / e->u, 1 / e->v); m_mul(e->phm2obj, t, e->phm2obj);

  int n = 0;
  double *x = NULL, *y = NULL;
  double radius, theta, start, stop;
  int cpts;
  switch (e->type) {
    case ORA_PELEM_RECTANGLE:
      n = 5; x = malloc(n * sizeof(double)); y = malloc(n * sizeof(double));
      x[0] = -e->u; y[0] = -e->v; x[1] = e->u; y[1] = -e->v; x[2] = e->u; y[2] = e->v;
      x[3] = -e->u; y[3] = e->v; x[4] = -e->u; y[4] = -e->v;
      break;
    case ORA_PELEM_TRIANGLE:
      n = 4; x = malloc(n * sizeof(double)); y = malloc(n * sizeof(double));
      x[0] = -e->u; y[0] = 0; x[1] = e->u; y[1] = 0; x[2] = 0; y[2] = e->v; x[3] = -e->u; y[3] = 0;
      break;
    case ORA_PELEM_ELLIPSE:
      n = circle_points(O_TWOPI);
      x = malloc(n * sizeof(double)); y = malloc(n * sizeof(double));
      arc_points(x, y, n, 0.0, 0.0, 1.0, 0.0, O_TWOPI);
      for (int i = 0; i < n; i++) { x[i] *= e->u; y[i] *= e->v; }
      break;
    case ORA_PELEM_SECTOR:
      radius = sqrt(e->u * e->u + e->v * e->v);
      theta = atan(e->u / e->v);
      start = 3.0 * O_HALFPI - theta; stop = 3.0 * O_HALFPI + theta;
      cpts = circle_points(stop - start);
      n = 3 + cpts; x = malloc(n * sizeof(double)); y = malloc(n * sizeof(double));
      x[0] = 0.0; y[0] = e->v; x[1] = -e->u; y[1] = 0.0;
      arc_points(&x[2], &y[2], cpts, 0.0, e->v, radius, start, stop);
      x[cpts + 2] = 0.0; y[cpts + 2] = e->v;
      break;
    case ORA_PELEM_SEGMENT:
      radius = sqrt(e->u * e->u + e->v * e->v);
      theta = atan(e->u / e->v);
      start = 3.0 * O_HALFPI - theta; stop = 3.0 * O_HALFPI + theta;
      cpts = circle_points(stop - start);
      n = cpts + 1; x = malloc(n * sizeof(double)); y = malloc(n * sizeof(double));
      arc_points(x, y, cpts, 0.0, e->v, radius, start, stop);
      x[cpts] = -e->u; y[cpts] = 0.0;
      break;
    default:
      return;
  }
  /* rotate2d / xlat2d: xform.cpp:33-64 */
  double c = cos(e->rot), s = sin(e->rot);
  for (int i = 0; i < n; i++) {
    double xr = x[i] * c - y[i] * s, yr = x[i] * s + y[i] * c;
    x[i] = xr + e->cx; y[i] = yr + e->cy;
  }
  e->xmin = e->xmax = x[0];
  e->ymin = e->ymax = y[0];
  for (int i = 1; i < n; i++) {
    if (x[i] < e->xmin) e->xmin = x[i]; else if (x[i] > e->xmax) e->xmax = x[i];
    if (y[i] < e->ymin) e->ymin = y[i]; else if (y[i] > e->ymax) e->ymax = y[i];
  }
  free(x); free(y);
}

int ora_phantom_init(ora_phantom* p, int maxElems) {
  memset(p, 0, sizeof(*p));
  p->cap = maxElems > 0 ? maxElems : 1;
  p->e = calloc((size_t)p->cap, sizeof(ora_pelem));
  p->xmin = 1E30; p->xmax = -1E30; p->ymin = 1E30; p->ymax = -1E30;   /* phantom.cpp:71-81 */
  return p->e != NULL;
}
void ora_phantom_free(ora_phantom* p) { free(p->e); p->e = NULL; p->n = 0; p->cap = 0; }

/* Phantom::addPElem: list push_front, limits union (phantom.cpp:237-256) */
int ora_phantom_add(ora_phantom* p, int type, double cx, double cy, double u, double v,
                    double rotDeg, double atten) {
  if (type == ORA_PELEM_INVALID) return 0;
  if (p->n >= p->cap) {   /* room for one more: double the array */
    const int cap = 2 * (p->cap > 0 ? p->cap : 1);
    ora_pelem* e = realloc(p->e, (size_t)cap * sizeof(ora_pelem));
    if (!e) return 0;
    p->e = e;
    p->cap = cap;
  }
  memmove(&p->e[1], &p->e[0], (size_t)p->n * sizeof(ora_pelem));
  ora_pelem* e = &p->e[0];
  memset(e, 0, sizeof(*e));
  e->type = type; e->cx = cx; e->cy = cy; e->u = u; e->v = v;
  e->rot = rotDeg * (O_PI / 180.); e->atten = atten;
  pelem_setup(e);
  if (p->xmin > e->xmin) p->xmin = e->xmin;
  if (p->xmax < e->xmax) p->xmax = e->xmax;
  if (p->ymin > e->ymin) p->ymin = e->ymin;
  if (p->ymax < e->ymax) p->ymax = e->ymax;
  p->n++;
  return 1;
}

/* built-in phantoms: phantom.cpp:144-170, :390-433 */
int ora_phantom_builtin(ora_phantom* p, const char* name) {
  static const double shepp[11][6] = {
    {0.0000, 0.0000, 0.6900, 0.9200, 0.0, 1.00},   {0.0000, -0.0184, 0.6624, 0.8740, 0.0, -0.98},
    {0.2200, 0.0000, 0.1100, 0.3100, -18.0, -0.02}, {-0.2200, 0.0000, 0.1600, 0.4100, 18.0, -0.02},
    {0.0000, 0.3500, 0.2100, 0.2500, 0.0, 0.01},    {0.0000, 0.1000, 0.0460, 0.0460, 0.0, 0.01},
    {0.0000, -0.1000, 0.0460, 0.0460, 0.0, 0.01},   {-0.0800, -0.6050, 0.0460, 0.0230, 0.0, 0.01},
    {0.0000, -0.6050, 0.0230, 0.0230, 0.0, 0.01},   {0.0600, -0.6050, 0.0230, 0.0230, 0.0, 0.01},
    {0.5538, -0.3858, 0.0330, 0.2060, -18.0, 0.03}};
  static const struct { int t; double a[6]; } herman[15] = {
    {ORA_PELEM_ELLIPSE, {0.000, 1.50, 0.375, 0.3000, 90.00, -0.003}},
    {ORA_PELEM_ELLIPSE, {0.675, -0.75, 0.225, 0.1500, 140.00, 0.010}},
    {ORA_PELEM_ELLIPSE, {0.750, 1.50, 0.375, 0.2250, 50.00, 0.003}},
    {ORA_PELEM_SEGMENT, {1.375, -7.50, 1.100, 0.6250, 19.20, -0.204}},
    {ORA_PELEM_SEGMENT, {1.375, -7.50, 1.100, 4.3200, 19.21, 0.204}},
    {ORA_PELEM_SEGMENT, {0.000, -2.25, 1.125, 0.3750, 0.00, -0.003}},
    {ORA_PELEM_SEGMENT, {0.000, -2.25, 1.125, 3.0000, 0.00, 0.003}},
    {ORA_PELEM_SEGMENT, {-1.000, 3.75, 1.000, 0.5000, 135.00, -0.003}},
    {ORA_PELEM_SEGMENT, {-1.000, 3.75, 1.000, 3.0000, 135.00, 0.003}},
    {ORA_PELEM_SEGMENT, {1.000, 3.75, 1.000, 0.5000, 225.00, -0.003}},
    {ORA_PELEM_SEGMENT, {1.000, 3.75, 1.000, 3.0000, 225.00, 0.003}},
    {ORA_PELEM_TRIANGLE, {5.025, 3.75, 1.125, 0.5000, 110.75, 0.206}},
    {ORA_PELEM_TRIANGLE, {-5.025, 3.75, 1.125, 0.9000, -110.75, 0.206}},
    {ORA_PELEM_ELLIPSE, {0.000, 0.00, 8.625, 6.4687, 90.00, 0.416}},
    {ORA_PELEM_ELLIPSE, {0.000, 0.00, 7.875, 5.7187, 90.00, -0.206}}};
  if (!strcasecmp(name, "shepp-logan")) {
    for (int i = 0; i < 11; i++)
      ora_phantom_add(p, ORA_PELEM_ELLIPSE, shepp[i][0], shepp[i][1], shepp[i][2], shepp[i][3],
                      shepp[i][4], shepp[i][5]);
    return 1;
  }
  if (!strcasecmp(name, "herman")) {
    for (int i = 0; i < 15; i++)
      ora_phantom_add(p, herman[i].t, herman[i].a[0], herman[i].a[1], herman[i].a[2],
                      herman[i].a[3], herman[i].a[4], herman[i].a[5]);
    return 1;
  }
  if (!strcasecmp(name, "unit-pulse")) {
    p->unit_pulse = 1;
    ora_phantom_add(p, ORA_PELEM_RECTANGLE, 0., 0., 100., 100., 0., 0.);
    ora_phantom_add(p, ORA_PELEM_ELLIPSE, 0., 0., 1., 1., 0., 1.);
    return 1;
  }
  return 0;
}

/* PhantomElement::clipLineWorldCoords + clipLineNormalizedCoords (phantom.cpp:830-898) */
static int pelem_clip(const ora_pelem* e, double* x1, double* y1, double* x2, double* y2) {
  double lim[4] = {e->xmin, e->ymin, e->xmax, e->ymax};
  double cx1 = *x1, cy1 = *y1, cx2 = *x2, cy2 = *y2;
  if (!clip_rect(&cx1, &cy1, &cx2, &cy2, lim)) return 0;
  m_apply(e->phm2obj, x1, y1);
  m_apply(e->phm2obj, x2, y2);
  int ok = 0;
  double unit[4] = {-1.0, -1.0, 1.0, 1.0};
  switch (e->type) {
    case ORA_PELEM_RECTANGLE: ok = clip_rect(x1, y1, x2, y2, unit); break;
    case ORA_PELEM_ELLIPSE: ok = clip_circle(x1, y1, x2, y2, 0.0, 0.0, 1.0, 0.0, 0.0); break;
    case ORA_PELEM_TRIANGLE: ok = clip_triangle(x1, y1, x2, y2, 1.0, 1.0, 1); break;
    case ORA_PELEM_SEGMENT: ok = clip_segment(x1, y1, x2, y2, e->u, e->v); break;
    case ORA_PELEM_SECTOR: ok = clip_sector(x1, y1, x2, y2, e->u, e->v); break;
    default: break;
  }
  if (!ok) return 0;
  m_apply(e->obj2phm, x1, y1);
  m_apply(e->obj2phm, x2, y2);
  return 1;
}

/* Scanner::projectSingleLine / projectLineAgainstPElem (scanner.cpp:611-656) */
double ora_raysum(const ora_phantom* p, double x1, double y1, double x2, double y2) {
  double sum = 0.0;
  for (int k = 0; k < p->n; k++) {
    double a = x1, b = y1, c = x2, d = y2;
    if (!pelem_clip(&p->e[k], &a, &b, &c, &d)) continue;
    double len = sqrt((c - a) * (c - a) + (d - b) * (d - b));   /* ctsupport.h:225 */
    sum += len * p->e[k].atten;
  }
  return sum;
}

/* ------------------------------------------------------------------------- */
/* Scanner geometry: libctsim/scanner.cpp:86-224                            */
/* ------------------------------------------------------------------------- */
int ora_geometry_id(const char* n) {
  if (!strcasecmp(n, "parallel")) return ORA_GEOM_PARALLEL;
  if (!strcasecmp(n, "equiangular")) return ORA_GEOM_EQUIANGULAR;
  if (!strcasecmp(n, "equilinear")) return ORA_GEOM_EQUILINEAR;
  return -1;
}

int ora_scanner_init(ora_scanner* s, const ora_phantom* p, int geometry, int nDet, int nView,
                     int offsetView, int nSample, double rotAngle, double flRatio,
                     double cdRatio, double viewRatio, double scanRatio) {
  memset(s, 0, sizeof(*s));
  if (geometry < 0 || geometry > 2 || nView < 1 || nDet < 1) { s->fail = 1; return 0; }
  s->geometry = geometry; s->nDet = nDet; s->nView = nView; s->offsetView = offsetView;
  s->nSample = nSample;
  double maxAxis = (p->xmax - p->xmin) > (p->ymax - p->ymin) ? (p->xmax - p->xmin)
                                                               : (p->ymax - p->ymin);
  s->viewDiameter = O_SQRT2 * maxAxis * viewRatio;        /* include/phantom.h:190-194 */
  s->focalLength = (s->viewDiameter / 2) * flRatio;
  s->centerDetectorLength = (s->viewDiameter / 2) * cdRatio;
  s->sourceDetectorLength = s->focalLength + s->centerDetectorLength;
  s->scanDiameter = s->viewDiameter * scanRatio;
  s->xCenter = p->xmin + (p->xmax - p->xmin) / 2;
  s->yCenter = p->ymin + (p->ymax - p->ymin) / 2;
  s->rotLen = rotAngle;
  s->rotInc = s->rotLen / nView;
  int even = (nDet % 2) == 0;
  if (geometry == ORA_GEOM_PARALLEL) {
    s->fanBeamAngle = 0;
    s->detLen = s->scanDiameter;
    s->detStart = -s->detLen / 2;
    s->detInc = s->detLen / nDet;
    double endOff = 0;
    if (even) { s->detInc = s->detLen / (nDet - 1); endOff = s->detInc; }
    double half = s->detLen / 2;
    s->xs1 = s->xCenter - half; s->ys1 = s->yCenter + s->focalLength;
    s->xs2 = s->xCenter + half + endOff; s->ys2 = s->yCenter + s->focalLength;
    s->xd1 = s->xCenter - half; s->yd1 = s->yCenter - s->centerDetectorLength;
    s->xd2 = s->xCenter + half + endOff; s->yd2 = s->yCenter - s->centerDetectorLength;
    s->detLen += endOff;
  } else if (geometry == ORA_GEOM_EQUILINEAR) {
    if (s->scanDiameter / 2 >= s->focalLength) { s->fail = 1; return 0; }
    double ang = asin((s->scanDiameter / 2) / s->focalLength);
    double half = s->sourceDetectorLength * tan(ang);
    s->detLen = half * 2;
    s->detStart = -half;
    s->detInc = s->detLen / nDet;
    double endOff = 0;
    if (even) { s->detInc = s->detLen / (nDet - 1); endOff = s->detInc; s->detLen += endOff; }
    s->fanBeamAngle = ang * 2;
    s->xs1 = s->xCenter; s->ys1 = s->yCenter + s->focalLength;
    s->xs2 = s->xCenter; s->ys2 = s->yCenter + s->focalLength;
    s->xd1 = s->xCenter - half; s->yd1 = s->yCenter - s->centerDetectorLength;
    s->xd2 = s->xCenter + half + endOff; s->yd2 = s->yCenter - s->centerDetectorLength;
  } else {
    if (s->scanDiameter / 2 > s->focalLength) { s->fail = 1; return 0; }
    double ang = asin((s->scanDiameter / 2) / s->focalLength);
    s->detLen = 2 * ang;
    s->detStart = -ang;
    s->detInc = s->detLen / nDet;
    double endOff = 0;
    if (even) { s->detInc = s->detLen / (nDet - 1); endOff = s->detInc; }
    double a1 = acos((s->scanDiameter / 2) / s->centerDetectorLength);
    double angScale = 2 * (O_HALFPI + ang - a1) / s->detLen;
    s->angularDetLen = angScale * (s->detLen + endOff);
    s->angularDetInc = angScale * s->detInc;
    s->fanBeamAngle = ang * 2;
    s->xs1 = s->xCenter; s->ys1 = s->yCenter + s->focalLength;
    s->xs2 = s->xCenter; s->ys2 = s->yCenter + s->focalLength;
    s->detLen += endOff;
  }
  mtx2 t;
  m_xlat(s->incmtx, -s->xCenter, -s->yCenter);
  m_rot(t, s->rotInc); m_mul(s->incmtx, t, s->incmtx);
  m_xlat(t, s->xCenter, s->yCenter); m_mul(s->incmtx, t, s->incmtx);
  return 1;
}

typedef struct { double xs1, ys1, xs2, ys2, xd1, yd1, xd2, yd2, angle; } view_pos;

/* Scanner::projectSingleView (scanner.cpp:445-533) */
static void project_view(const ora_scanner* s, const ora_phantom* p, const view_pos* vp,
                         double* det) {
  int nDet = s->nDet, nSample = s->nSample;
  if (p->unit_pulse) {
    for (int d = 0; d < nDet; d++) det[d] = 0;
    det[nDet / 2] = 1;
    return;
  }
  double sdx = (vp->xs2 - vp->xs1) / nDet, sdy = (vp->ys2 - vp->ys1) / nDet;
  double xs_maj = vp->xs1 + (sdx / 2), ys_maj = vp->ys1 + (sdy / 2);
  double ddx = 0, ddy = 0, ddx2 = 0, ddy2 = 0, xd_maj = 0, yd_maj = 0;
  double angInc = 0, angSampleInc = 0, angMajor = 0;
  double detAngle = vp->angle + 3 * O_HALFPI;
  if (s->geometry == ORA_GEOM_EQUIANGULAR) {
    angInc = s->angularDetInc;
    angSampleInc = angInc / nSample;
    angMajor = detAngle - (s->angularDetLen / 2) + angSampleInc / 2;
  } else {
    ddx = (vp->xd2 - vp->xd1) / nDet; ddy = (vp->yd2 - vp->yd1) / nDet;
    ddx2 = ddx / nSample; ddy2 = ddy / nSample;
    xd_maj = vp->xd1 + ddx2 / 2; yd_maj = vp->yd1 + ddy2 / 2;
  }
  for (int d = 0; d < nDet; d++) {
    double xs = xs_maj, ys = ys_maj, xd = 0, yd = 0, ang = 0;
    if (s->geometry == ORA_GEOM_EQUIANGULAR) ang = angMajor;
    else { xd = xd_maj; yd = yd_maj; }
    double sum = 0.0;
    for (int i = 0; i < nSample; i++) {
      if (s->geometry == ORA_GEOM_EQUIANGULAR) {
        xd = s->centerDetectorLength * cos(ang);
        yd = s->centerDetectorLength * sin(ang);
      }
      sum += ora_raysum(p, xd, yd, xs, ys);
      if (s->geometry == ORA_GEOM_EQUIANGULAR) ang += angSampleInc;
      else { xd += ddx2; yd += ddy2; }
    }
    det[d] = sum / nSample;
    xs_maj += sdx; ys_maj += sdy;
    if (s->geometry == ORA_GEOM_EQUIANGULAR) angMajor += angInc;
    else { xd_maj += ddx; yd_maj += ddy; }
  }
}

/* Scanner::collectProjections (scanner.cpp:295-419).  The endpoint positions of
 * every view are produced by the reference's sequential incremental rotation
 * first; the views are then ray-traced in parallel. */
void ora_collect_projections(const ora_scanner* s, const ora_phantom* p, int iStartView,
                             int iNumViews, int iOffsetView, int iStorageOffset, double* sino,
                             double* viewAngles, int nThreads) {
  if (iNumViews <= 0) return;
  view_pos* vp = malloc((size_t)iNumViews * sizeof(view_pos));
  double start = (iStartView + iOffsetView) * s->rotInc;
  mtx2 m0, t;
  m_xlat(m0, -s->xCenter, -s->yCenter);
  m_rot(t, start); m_mul(m0, t, m0);
  m_xlat(t, s->xCenter, s->yCenter); m_mul(m0, t, m0);
  double xd1 = 0, yd1 = 0, xd2 = 0, yd2 = 0;
  if (s->geometry != ORA_GEOM_EQUIANGULAR) {
    xd1 = s->xd1; yd1 = s->yd1; xd2 = s->xd2; yd2 = s->yd2;
    m_apply((const double(*)[3])m0, &xd1, &yd1);
    m_apply((const double(*)[3])m0, &xd2, &yd2);
  }
  double xs1 = s->xs1, ys1 = s->ys1, xs2 = s->xs2, ys2 = s->ys2;
  m_apply((const double(*)[3])m0, &xs1, &ys1);
  m_apply((const double(*)[3])m0, &xs2, &ys2);
  double ang = start;
  for (int v = 0; v < iNumViews; v++, ang += s->rotInc) {
    view_pos q = {xs1, ys1, xs2, ys2, xd1, yd1, xd2, yd2, ang};
    vp[v] = q;
    m_apply(s->incmtx, &xs1, &ys1);
    m_apply(s->incmtx, &xs2, &ys2);
    if (s->geometry != ORA_GEOM_EQUIANGULAR) {
      m_apply(s->incmtx, &xd1, &yd1);
      m_apply(s->incmtx, &xd2, &yd2);
    }
  }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nThreads > 0 ? nThreads : 1)
  for (int v = 0; v < iNumViews; v++) {
    int row = v + iStorageOffset;
    project_view(s, p, &vp[v], &sino[(size_t)row * s->nDet]);
    if (viewAngles) viewAngles[row] = vp[v].angle;
  }
  free(vp);
}

/* Gradient of sum_{v,d} gsino[v][d] sino[v][d] with respect to the ellipse
 * parameters (cx, cy, u, v, rot radians, atten) of every element (list
 * order), FP64.  No reference counterpart: the derivative of the chord
 * c = 2 u v sqrt(Q - rho^2) / Q, Q = v^2 ra^2 + u^2 rb^2, of each ray that
 * projectSingleView (scanner.cpp:445-533) traces and the element's outline
 * box accepts (scanner.cpp:611-656 with phantom.cpp:830-850), the box held
 * fixed.  Views as ora_collect_projections over all views. */
static void ray_grad(const ora_phantom* p, double xd, double yd, double xs, double ys, double w,
                     double* grad) {
  double dx = xd - xs, dy = yd - ys, n = 1.0 / sqrt(dx * dx + dy * dy);
  double rx = dx * n, ry = dy * n;
  for (int k = 0; k < p->n; k++) {
    const ora_pelem* e = &p->e[k];
    if (e->type != ORA_PELEM_ELLIPSE) continue;
    double ct = cos(e->rot), st = sin(e->rot), u = e->u, v = e->v;
    double rho = rx * (e->cy - ys) - ry * (e->cx - xs);
    double ra = rx * ct + ry * st, rb = -rx * st + ry * ct;
    double Q = v * v * ra * ra + u * u * rb * rb, h2 = Q - rho * rho;
    if (!(h2 > 0.0)) continue;
    double lim[4] = {e->xmin, e->ymin, e->xmax, e->ymax};
    double x1 = xd, y1 = yd, x2 = xs, y2 = ys;
    if (!clip_rect(&x1, &y1, &x2, &y2, lim)) continue;
    double hc = sqrt(h2), iQ = 1.0 / Q, c = 2.0 * u * v * hc * iQ;
    double dcdrho = -2.0 * u * v * rho * iQ / hc;
    double dcdQ = u * v * (2.0 * rho * rho - Q) * iQ * iQ / hc;
    double ga = w * e->atten, *g = grad + 6 * k;
    g[0] += ga * dcdrho * -ry;
    g[1] += ga * dcdrho * rx;
    g[2] += ga * (2.0 * v * hc * iQ + dcdQ * 2.0 * u * rb * rb);
    g[3] += ga * (2.0 * u * hc * iQ + dcdQ * 2.0 * v * ra * ra);
    g[4] += ga * dcdQ * 2.0 * ra * rb * (v * v - u * u);
    g[5] += w * c;
  }
}

void ora_ellipse_gradient(const ora_scanner* s, const ora_phantom* p, const double* gsino,
                          double* grad) {
  int nv = s->nView, nDet = s->nDet, nSample = s->nSample;
  for (int i = 0; i < 6 * p->n; i++) grad[i] = 0;
  mtx2 m0, t;
  m_xlat(m0, -s->xCenter, -s->yCenter);
  m_rot(t, s->offsetView * s->rotInc); m_mul(m0, t, m0);
  m_xlat(t, s->xCenter, s->yCenter); m_mul(m0, t, m0);
  double xd1 = 0, yd1 = 0, xd2 = 0, yd2 = 0;
  if (s->geometry != ORA_GEOM_EQUIANGULAR) {
    xd1 = s->xd1; yd1 = s->yd1; xd2 = s->xd2; yd2 = s->yd2;
    m_apply((const double(*)[3])m0, &xd1, &yd1);
    m_apply((const double(*)[3])m0, &xd2, &yd2);
  }
  double xs1 = s->xs1, ys1 = s->ys1, xs2 = s->xs2, ys2 = s->ys2;
  m_apply((const double(*)[3])m0, &xs1, &ys1);
  m_apply((const double(*)[3])m0, &xs2, &ys2);
  double ang = s->offsetView * s->rotInc;
  for (int vi = 0; vi < nv; vi++, ang += s->rotInc) {
    /* the rays of projectSingleView for this view */
    double sdx = (xs2 - xs1) / nDet, sdy = (ys2 - ys1) / nDet;
    double xs_maj = xs1 + (sdx / 2), ys_maj = ys1 + (sdy / 2);
    double ddx = 0, ddy = 0, ddx2 = 0, ddy2 = 0, xd_maj = 0, yd_maj = 0;
    double angInc = 0, angSampleInc = 0, angMajor = 0;
    if (s->geometry == ORA_GEOM_EQUIANGULAR) {
      angInc = s->angularDetInc;
      angSampleInc = angInc / nSample;
      angMajor = ang + 3 * O_HALFPI - (s->angularDetLen / 2) + angSampleInc / 2;
    } else {
      ddx = (xd2 - xd1) / nDet; ddy = (yd2 - yd1) / nDet;
      ddx2 = ddx / nSample; ddy2 = ddy / nSample;
      xd_maj = xd1 + ddx2 / 2; yd_maj = yd1 + ddy2 / 2;
    }
    for (int d = 0; d < nDet; d++) {
      double xs = xs_maj, ys = ys_maj, xd = 0, yd = 0, a = 0;
      if (s->geometry == ORA_GEOM_EQUIANGULAR) a = angMajor;
      else { xd = xd_maj; yd = yd_maj; }
      double w = gsino[(size_t)vi * nDet + d] / nSample;
      for (int i = 0; i < nSample; i++) {
        if (s->geometry == ORA_GEOM_EQUIANGULAR) {
          xd = s->centerDetectorLength * cos(a);
          yd = s->centerDetectorLength * sin(a);
        }
        ray_grad(p, xd, yd, xs, ys, w, grad);
        if (s->geometry == ORA_GEOM_EQUIANGULAR) a += angSampleInc;
        else { xd += ddx2; yd += ddy2; }
      }
      xs_maj += sdx; ys_maj += sdy;
      if (s->geometry == ORA_GEOM_EQUIANGULAR) angMajor += angInc;
      else { xd_maj += ddx; yd_maj += ddy; }
    }
    m_apply(s->incmtx, &xs1, &ys1);
    m_apply(s->incmtx, &xs2, &ys2);
    if (s->geometry != ORA_GEOM_EQUIANGULAR) {
      m_apply(s->incmtx, &xd1, &yd1);
      m_apply(s->incmtx, &xd2, &yd2);
    }
  }
}

/* Helical scan of a 3-D ellipsoid phantom: a restatement with no reference
 * counterpart (CTSim's phantoms are 2-D).  View v of the scanner (positions
 * as collectProjections over all views, scanner.cpp:295-419) sees the
 * phantom's cross-section at z = z0 + v dz: ellipsoid k (cx, cy, cz, a, b, c,
 * rotation about z in degrees, attenuation) contributes the ellipse
 * (cx, cy, a s, b s) with s = sqrt(1 - ((z - cz)/c)^2) when |z - cz| < c,
 * added in ellipsoid order (so the list order is the reference's, last
 * added first), and the view is projected as projectSingleView does. */
void ora_collect_ellipsoids(const ora_scanner* s, const double* ell, int n, double z0, double dz,
                            double* sino, double* viewAngles, int nThreads) {
  int nv = s->nView;
  view_pos* vp = malloc((size_t)nv * sizeof(view_pos));
  double start = 0.0;
  mtx2 m0, t;
  m_xlat(m0, -s->xCenter, -s->yCenter);
  m_rot(t, start); m_mul(m0, t, m0);
  m_xlat(t, s->xCenter, s->yCenter); m_mul(m0, t, m0);
  double xd1 = 0, yd1 = 0, xd2 = 0, yd2 = 0;
  if (s->geometry != ORA_GEOM_EQUIANGULAR) {
    xd1 = s->xd1; yd1 = s->yd1; xd2 = s->xd2; yd2 = s->yd2;
    m_apply((const double(*)[3])m0, &xd1, &yd1);
    m_apply((const double(*)[3])m0, &xd2, &yd2);
  }
  double xs1 = s->xs1, ys1 = s->ys1, xs2 = s->xs2, ys2 = s->ys2;
  m_apply((const double(*)[3])m0, &xs1, &ys1);
  m_apply((const double(*)[3])m0, &xs2, &ys2);
  double ang = start;
  for (int v = 0; v < nv; v++, ang += s->rotInc) {
    view_pos q = {xs1, ys1, xs2, ys2, xd1, yd1, xd2, yd2, ang};
    vp[v] = q;
    m_apply(s->incmtx, &xs1, &ys1);
    m_apply(s->incmtx, &xs2, &ys2);
    if (s->geometry != ORA_GEOM_EQUIANGULAR) {
      m_apply(s->incmtx, &xd1, &yd1);
      m_apply(s->incmtx, &xd2, &yd2);
    }
  }
#pragma omp parallel for schedule(dynamic, 4) num_threads(nThreads > 0 ? nThreads : 1)
  for (int v = 0; v < nv; v++) {
    ora_phantom p;
    ora_phantom_init(&p, n > 0 ? n : 1);
    double z = z0 + v * dz;
    for (int k = 0; k < n; k++) {
      const double* e = ell + 8 * k;
      double d = (z - e[2]) / e[5];
      if (!(fabs(d) < 1.0)) continue;
      double sc = sqrt((1.0 - d) * (1.0 + d));
      ora_phantom_add(&p, ORA_PELEM_ELLIPSE, e[0], e[1], e[3] * sc, e[4] * sc, e[6], e[7]);
    }
    project_view(s, &p, &vp[v], &sino[(size_t)v * s->nDet]);
    if (viewAngles) viewAngles[v] = vp[v].angle;
    ora_phantom_free(&p);
  }
  free(vp);
}

/* ------------------------------------------------------------------------- */
/* Signal filters: libctsim/filter.cpp                                      */
/* ------------------------------------------------------------------------- */
enum { F_ABS_BANDLIMIT = 0, F_ABS_G_HAMMING, F_ABS_HANNING, F_ABS_COSINE, F_ABS_SINC, F_SHEPP,
       F_BANDLIMIT, F_SINC, F_G_HAMMING, F_HANNING, F_COSINE, F_TRIANGLE };

/* name table is NOT in ID order: filter.cpp:30-59 ("shepp" -> 4, "abs_sinc" -> 5) */
int ora_filter_id(const char* n) {
  static const char* names[12] = {"abs_bandlimit", "abs_hamming", "abs_hanning", "abs_cosine",
                                  "shepp", "abs_sinc", "bandlimit", "sinc", "hamming",
                                  "hanning", "cosine", "triangle"};
  for (int i = 0; i < 12; i++)
    if (!strcasecmp(n, names[i])) return i;
  return -1;
}
int ora_filter_method_id(const char* n) {   /* procsignal.cpp:42-51 */
  if (!strcasecmp(n, "convolution")) return ORA_FM_CONVOLUTION;
  if (!strcasecmp(n, "fourier")) return ORA_FM_FOURIER;
  if (!strcasecmp(n, "fouier-table")) return ORA_FM_FOURIER_TABLE;
  if (!strcasecmp(n, "fft")) return ORA_FM_FFT;
  return -1;
}
int ora_filter_generation_id(const char* n) {   /* procsignal.cpp:68-71 */
  if (!strcasecmp(n, "direct")) return ORA_FG_DIRECT;
  if (!strcasecmp(n, "inverse-fourier")) return ORA_FG_INVERSE_FOURIER;
  return -1;
}

/* include/filter.h:120-124, :163-164 */
static double sinc1(double x) { return fabs(x) > O_FEPS ? sin(x) / x : 1.0; }
static double sinc2(double x, double m) { return fabs(x) > O_FEPS ? sin(x * m) / x : 1.0; }
static double int_abscos(double u, double w) {
  return fabs(u) > O_FEPS ? (cos(u * w) - 1) / (u * u) + w / u * sin(u * w) : (w * w / 2);
}

/* SignalFilter::frequencyResponse (filter.cpp:403-475) */
double ora_frequency_response(int id, double bw, double u, double param) {
  double q, au = fabs(u), abw = fabs(bw);
  int outside = au >= (abw / 2) + O_FEPS;
  switch (id) {
    case F_BANDLIMIT: q = outside ? 0. : 1; break;
    case F_ABS_BANDLIMIT: q = outside ? 0. : au; break;
    case F_TRIANGLE: q = outside ? 0 : 1 - au / abw; break;
    case F_COSINE: q = outside ? 0 : cos(O_PI * au / abw); break;
    case F_ABS_COSINE: q = outside ? 0 : au * cos(O_PI * au / abw); break;
    case F_SINC: q = abw * sinc2(O_PI * abw * au, 1.); break;
    case F_ABS_SINC: q = outside ? 0 : au * abw * sinc2(O_PI * abw * au, 1.); break;
    case F_HANNING: param = 0.5; /* fall through */
    case F_G_HAMMING: q = outside ? 0 : param + (1 - param) * cos(O_TWOPI * au / abw); break;
    case F_ABS_HANNING: param = 0.5; /* fall through */
    case F_ABS_G_HAMMING:
      q = outside ? 0 : au * (param + (1 - param) * cos(O_TWOPI * au / abw));
      break;
    default: q = 0; break;
  }
  return q;
}

/* filter.cpp:499-523 */
static int have_analytic(int id) {
  return id == F_BANDLIMIT || id == F_TRIANGLE || id == F_COSINE || id == F_G_HAMMING ||
         id == F_HANNING || id == F_ABS_BANDLIMIT || id == F_ABS_COSINE ||
         id == F_ABS_G_HAMMING || id == F_ABS_HANNING || id == F_SHEPP || id == F_SINC;
}
/* filter.cpp:525-584 */
static double spatial_analytic(int id, double bw, double x, double param) {
  double q, temp, u = O_TWOPI * x, w = bw / 2, b = O_PI / bw, b2 = O_TWOPI / bw;
  switch (id) {
    case F_BANDLIMIT: q = bw * sinc2(u * w, 1.0); break;
    case F_TRIANGLE: temp = sinc2(u * w, 1.0); q = bw * temp * temp; break;
    case F_COSINE: q = sinc2(b - u, w) + sinc2(b + u, w); break;
    case F_HANNING: param = 0.5; /* fall through */
    case F_G_HAMMING:
      q = 2 * param * sin(u * w) / u + (1 - param) * (sinc2(b2 - u, w) + sinc2(b2 + u, w));
      break;
    case F_ABS_BANDLIMIT: q = 2 * int_abscos(u, w); break;
    case F_ABS_COSINE: q = int_abscos(b - u, w) + int_abscos(b + u, w); break;
    case F_ABS_HANNING: param = 0.5; /* fall through */
    case F_ABS_G_HAMMING:
      q = 2 * param * int_abscos(u, w) + (1 - param) * (int_abscos(u - b2, w) + int_abscos(u + b2, w));
      break;
    case F_SHEPP:
      if (fabs(u) < 1E-7) q = 4. / (O_PI * bw * bw);
      else q = fabs((2 / bw) * sin(u * w)) * sinc2(u * w, 1.) * sinc2(u * w, 1.);
      break;
    case F_SINC: q = fabs(x) < bw / 2 ? 1. : 0.; break;
    default: q = 0; break;
  }
  return q;
}
/* Simpson integration: libctsupport/mathfuncs.cpp:37-67 */
static double simpson(double xmin, double xmax, const double* y, int np) {
  if (np < 2) return 0.;
  if (np == 2) return (xmax - xmin) * (y[0] + y[1]) / 2;
  double area = 0;
  int nDiv = (np - 1) / 2;
  double width = (xmax - xmin) / (double)(np - 1);
  for (int i = 1; i <= nDiv; i++) {
    int xr = 2 * i, xl = xr - 2, xm = xr - 1;
    area += (width / 3.0) * (y[xl] + 4.0 * y[xm] + y[xr]);
  }
  if ((np & 1) == 0) area += width * (y[np - 2] + y[np - 1]) / 2;
  return area;
}
/* numeric inverse transform, N_INTEGRAL = 500: filter.cpp:28, :358-381 */
static double spatial_calc(int id, double bw, double x, double param) {
  const int n = 500;
  double zmin = 0, zmax = (id == F_TRIANGLE) ? bw : bw / 2;
  double zinc = (zmax - zmin) / (n - 1), z = zmin;
  double q[500];
  for (int i = 0; i < n; i++, z += zinc)
    q[i] = ora_frequency_response(id, bw, z, param) * cos(O_TWOPI * z * x);
  return 2 * simpson(zmin, zmax, q, n);
}
double ora_spatial_response(int id, double bw, double x, double param) {
  return have_analytic(id) ? spatial_analytic(id, bw, x, param) : spatial_calc(id, bw, x, param);
}

/* SignalFilter::init + create{Frequency,Spatial}Filter (filter.cpp:158-229) */
static void make_filter(int id, double fmin, double fmax, int n, double bw, double param,
                        int spatial, double* out) {
  double inc = (fmax - fmin) / (n - 1);
  if (!spatial) {
    double x = fmin;
    for (int i = 0; i < n; i++, x += inc) out[i] = ora_frequency_response(id, bw, x, param);
    return;
  }
  if (id == F_SHEPP) {
    double a = 2 * bw, c = -4. / (a * a);
    int center = (n - 1) / 2;
    out[center] = 4. / (a * a);
    for (int i = 1; i <= center; i++) out[center + i] = out[center - i] = c / (4 * (i * i) - 1);
  } else {
    double x = fmin;
    for (int i = 0; i < n; i++, x += inc) out[i] = ora_spatial_response(id, bw, x, param);
  }
}

/* include/fourier.h:50-100 */
static void natural_to_fourier(double* v, int n) {
  double* t = malloc((size_t)n * sizeof(double));
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
  memcpy(v, t, (size_t)n * sizeof(double));
  free(t);
}
static void fourier_to_natural(double* v, int n) {
  double* t = malloc((size_t)n * sizeof(double));
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
  memcpy(v, t, (size_t)n * sizeof(double));
  free(t);
}

/* O(n^2) transforms: procsignal.cpp:694-774.  The direction constants are
 * FORWARD = -1 (which also divides by n) and BACKWARD = +1 (include/procsignal.h:62-63). */
#define O_FORWARD (-1)
#define O_BACKWARD 1
static void dft_r2c(const double* in, double* re, double* im, int n, int dir) {
  dir = dir < 0 ? -1 : 1;
  double ai = dir * 2 * O_PI / n;
  for (int i = 0; i < n; i++) {
    double sr = 0, si = 0;
    for (int j = 0; j < n; j++) {
      double a = i * j * ai;
      sr += in[j] * cos(a);
      si += in[j] * sin(a);
    }
    if (dir < 0) { sr /= n; si /= n; }
    re[i] = sr; im[i] = si;
  }
}
static void dft_c2r(const double* re, const double* im, double* out, int n, int dir) {
  dir = dir < 0 ? -1 : 1;
  double ai = dir * 2 * O_PI / n;
  for (int i = 0; i < n; i++) {
    double sr = 0;
    for (int j = 0; j < n; j++) {
      double a = i * j * ai;
      sr += re[j] * cos(a) - im[j] * sin(a);
    }
    if (dir < 0) sr /= n;
    out[i] = sr;
  }
}

/* addZeropadFactor: procsignal.cpp:867-881 */
static int zeropad_size(int n, int z) {
  if (z > 0) {
    double l2 = log(n) / log(2);
    int il = (int)floor(l2);
    return 1 << (il + z);
  }
  return n;
}

/* ProcessSignal::init (procsignal.cpp:123-442) */
int ora_procsig_init(ora_procsig* ps, int filterId, int method, double bandwidth,
                     double signalInc, int nSignal, double param, int generation, int zeropad,
                     int interpFactor, int geometry, double focalLength, double sdl) {
  memset(ps, 0, sizeof(*ps));
  if (filterId < 0 || method < 0 || generation < 0) { ps->fail = 1; return 0; }
  ps->filterId = filterId; ps->method = method; ps->generation = generation;
  ps->geometry = geometry; ps->focalLength = focalLength; ps->sdl = sdl;
  ps->bandwidth = bandwidth; ps->nSignal = nSignal; ps->signalInc = signalInc;
  ps->param = param; ps->zeropad = zeropad; ps->interpFactor = interpFactor;
  if (geometry == ORA_GEOM_EQUILINEAR) {
    double scale = sdl / focalLength;
    ps->signalInc /= scale;
    ps->bandwidth *= scale;
  }
  double inc = ps->signalInc, bw = ps->bandwidth;
  int n = nSignal;
  if (method == ORA_FM_CONVOLUTION) {
    ps->nFilterPoints = 2 * (n - 1) + 1;
    int nf = ps->nFilterPoints;
    ps->filter = malloc((size_t)nf * sizeof(double));
    if (generation == ORA_FG_DIRECT) {
      double fmin = -inc * (n - 1), fmax = inc * (n - 1);
      make_filter(filterId, fmin, fmax, nf, bw, param, 1, ps->filter);
    } else {
      double fmin = -1. / (2 * inc), fmax = 1. / (2 * inc);
      double* freq = malloc((size_t)nf * sizeof(double));
      make_filter(filterId, fmin, fmax, nf, bw, param, 0, freq);
      natural_to_fourier(freq, nf);
      double* im = malloc((size_t)nf * sizeof(double));
      dft_r2c(freq, ps->filter, im, nf, O_FORWARD);
      free(im); free(freq);
      fourier_to_natural(ps->filter, nf);
      for (int i = 0; i < nf; i++) ps->filter[i] /= inc;
    }
    if (geometry == ORA_GEOM_EQUILINEAR) {
      for (int i = 0; i < nf; i++) ps->filter[i] *= 0.5;
    } else if (geometry == ORA_GEOM_EQUIANGULAR) {
      for (int i = 0; i < nf; i++) {
        int k = i - ((nf - 1) / 2);
        double ss = 1 / sinc1(k * inc);
        ps->filter[i] *= 0.5 * ss * ss;
      }
    }
  } else {
    if (generation == ORA_FG_DIRECT) {
      ps->nFilterPoints = zeropad_size(n, zeropad);
      int nf = ps->nFilterPoints;
      ps->nOutput = nf * interpFactor;
      double fmin = -1. / (2 * inc), fmax = 1. / (2 * inc), finc;
      if (nf % 2) finc = (fmax - fmin) / (nf - 1);
      else { finc = (fmax - fmin) / nf; fmax -= finc; }
      (void)finc;
      ps->filter = malloc((size_t)nf * sizeof(double));
      make_filter(filterId, fmin, fmax, nf, bw, param, 0, ps->filter);
      if (geometry == ORA_GEOM_EQUILINEAR) {
        for (int i = 0; i < nf; i++) ps->filter[i] *= 0.5;
      } else if (geometry == ORA_GEOM_EQUIANGULAR) {
        for (int i = 0; i < nf; i++) {
          int k = i - ((nf - 1) / 2);
          double ss = 1 / sinc1(k * inc);
          ps->filter[i] *= 0.5 * ss * ss;
        }
      }
      natural_to_fourier(ps->filter, nf);
    } else {
      int nsp = 2 * (n - 1) + 1;
      double fmin = -inc * (n - 1), fmax = inc * (n - 1);
      int nf = nsp;
      if (zeropad > 0) {
        double l2 = log(nsp) / log(2);
        int np2 = (int)floor(l2);
        if (l2 != floor(l2)) np2++;
        np2 += zeropad - 1;
        nf = 1 << np2;
      }
      ps->nFilterPoints = nf;
      ps->nOutput = nf * interpFactor;
      double* sp = calloc((size_t)(nf > nsp ? nf : nsp), sizeof(double));
      make_filter(filterId, fmin, fmax, nsp, bw, param, 1, sp);
      if (geometry == ORA_GEOM_EQUILINEAR) {
        for (int i = 0; i < nsp; i++) sp[i] *= 0.5;
      } else if (geometry == ORA_GEOM_EQUIANGULAR) {
        for (int i = 0; i < nsp; i++) {
          int k = i - ((nsp - 1) / 2);
          double ss = sin(k * inc);
          ss = fabs(ss) < 1E-7 ? 1 : (k * inc) / ss;
          sp[i] *= 0.5 * ss * ss;
        }
      }
      for (int i = nsp; i < nf; i++) sp[i] = 0;
      ps->filter = malloc((size_t)nf * sizeof(double));
      double* re = malloc((size_t)nf * sizeof(double));
      double* im = malloc((size_t)nf * sizeof(double));
      dft_r2c(sp, re, im, nf, O_BACKWARD);
      for (int i = 0; i < nf; i++) ps->filter[i] = hypot(re[i], im[i]) * inc;
      free(re); free(im); free(sp);
    }
    if (method == ORA_FM_FOURIER_TABLE) {   /* procsignal.cpp:399-410 */
      int m = ps->nFilterPoints > ps->nOutput ? ps->nFilterPoints : ps->nOutput;
      ps->nTable = m * m + 1;
      ps->cosTable = malloc((size_t)ps->nTable * sizeof(double));
      ps->sinTable = malloc((size_t)ps->nTable * sizeof(double));
      double ai = (2. * O_PI) / ps->nFilterPoints, a = 0;
      for (int i = 0; i < ps->nTable; i++) {
        ps->cosTable[i] = cos(a);
        ps->sinTable[i] = sin(a);
        a += ai;
      }
    }
  }
  return 1;
}

void ora_procsig_free(ora_procsig* ps) {
  free(ps->filter); free(ps->cosTable); free(ps->sinTable);
  memset(ps, 0, sizeof(*ps));
}

/* In-place radix-2 complex FFT of length n (a power of two), exp(sign*2*pi*i*jk/n),
 * Cooley-Tukey decimation in time.  Used for the "fft" method, whose reference
 * path (FFTW's R2HC / HC2R, procsignal.cpp:600-613) computes the same product
 * as the O(n^2) "fourier" method. */
static void fft_pow2(double* re, double* im, int n, int sign) {
  for (int i = 1, j = 0; i < n; i++) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double t = re[i]; re[i] = re[j]; re[j] = t;
      t = im[i]; im[i] = im[j]; im[j] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    double ang = sign * 2 * O_PI / len;
    for (int i = 0; i < n; i += len) {
      for (int k = 0; k < len / 2; k++) {
        double wr = cos(ang * k), wi = sin(ang * k);
        int a = i + k, b = i + k + len / 2;
        double xr = re[b] * wr - im[b] * wi, xi = re[b] * wi + im[b] * wr;
        re[b] = re[a] - xr; im[b] = im[a] - xi;
        re[a] += xr; im[a] += xi;
      }
    }
  }
}

/* ProcessSignal::filterSignal (procsignal.cpp:543-629) */
void ora_filter_signal(const ora_procsig* ps, const float* cin, double* out) {
  int n = ps->nSignal, nf = ps->nFilterPoints;
  double* in = malloc((size_t)n * sizeof(double));
  for (int i = 0; i < n; i++) in[i] = cin[i];
  double fl = ps->focalLength, inc = ps->signalInc;
  if (ps->geometry == ORA_GEOM_EQUILINEAR) {
    for (int i = 0; i < n; i++) {
      int k = i - (n / 2);
      in[i] *= fl / sqrt(fl * fl + k * k * inc * inc);
    }
  } else if (ps->geometry == ORA_GEOM_EQUIANGULAR) {
    for (int i = 0; i < n; i++) {
      int k = i - (n / 2);
      in[i] *= fl * cos(k * inc);
    }
  }
  if (ps->method == ORA_FM_CONVOLUTION) {   /* convolve: procsignal.cpp:658-691 */
    for (int i = 0; i < n; i++) {
      double sum = 0.0;
      const double* f2 = ps->filter + i + (n - 1);
      for (int j = 0; j < n; j++) sum += in[j] * *f2--;
      out[i] = sum * inc;
    }
  } else if (ps->method == ORA_FM_FOURIER || ps->method == ORA_FM_FFT) {
    double* x = calloc((size_t)nf, sizeof(double));
    double* re = malloc((size_t)nf * sizeof(double));
    double* im = malloc((size_t)nf * sizeof(double));
    for (int i = 0; i < n; i++) x[i] = in[i];
    if (ps->method == ORA_FM_FFT && (nf & (nf - 1)) == 0) {
      /* FFTW: unnormalised forward R2HC, filter divided by n, unnormalised HC2R */
      for (int i = 0; i < nf; i++) { re[i] = x[i]; im[i] = 0; }
      fft_pow2(re, im, nf, -1);
      for (int i = 0; i < nf; i++) {
        double h = ps->filter[i] / nf;
        re[i] *= h; im[i] *= h;
      }
      fft_pow2(re, im, nf, +1);
      for (int i = 0; i < n; i++) out[i] = re[i];
    } else {
      dft_r2c(x, re, im, nf, O_FORWARD);
      for (int i = 0; i < nf; i++) { re[i] *= ps->filter[i]; im[i] *= ps->filter[i]; }
      double* inv = malloc((size_t)nf * sizeof(double));
      dft_c2r(re, im, inv, nf, O_BACKWARD);
      for (int i = 0; i < n; i++) out[i] = inv[i];
      free(inv);
    }
    free(x); free(re); free(im);
  } else if (ps->method == ORA_FM_FOURIER_TABLE) {   /* procsignal.cpp:778-864 */
    double* x = calloc((size_t)nf, sizeof(double));
    double* re = malloc((size_t)nf * sizeof(double));
    double* im = malloc((size_t)nf * sizeof(double));
    for (int i = 0; i < n; i++) x[i] = in[i];
    for (int i = 0; i < nf; i++) {   /* FORWARD: minus sine, divide by n */
      double sr = 0, si = 0;
      for (int j = 0; j < nf; j++) {
        int t = i * j;
        sr += x[j] * ps->cosTable[t];
        si -= x[j] * ps->sinTable[t];
      }
      sr /= nf; si /= nf;
      re[i] = sr * ps->filter[i]; im[i] = si * ps->filter[i];
    }
    for (int i = 0; i < n; i++) {    /* BACKWARD, real part */
      double sr = 0;
      for (int j = 0; j < nf; j++) {
        int t = i * j;
        sr += re[j] * ps->cosTable[t] - im[j] * ps->sinTable[t];
      }
      out[i] = sr;
    }
    free(x); free(re); free(im);
  }
  free(in);
}

void ora_filter_views(const ora_procsig* ps, const float* sino, int nView, double* out,
                      int nThreads) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nThreads > 0 ? nThreads : 1)
  for (int v = 0; v < nView; v++)
    ora_filter_signal(ps, &sino[(size_t)v * ps->nSignal], &out[(size_t)v * ps->nSignal]);
}

/* ------------------------------------------------------------------------- */
/* Backprojectors: libctsim/backprojectors.cpp                              */
/* ------------------------------------------------------------------------- */
/* CubicPolyInterpolator::interpolate (libctsupport/interpolator.cpp:37-75) */
double ora_cubic_interpolate(const double* y, int n, double x) {
  int lo = (int)floor(x) - 1, hi = lo + 3;
  if (lo < -1) return 0;
  if (lo == -1) return y[0] + x * (y[1] - y[0]);
  if (hi > n) return 0;
  if (hi == n) {
    double frac = x - (lo + 1);
    return y[n - 2] + frac * (y[n - 1] - y[n - 2]);
  }
  double d0 = x - lo, d1 = x - (lo + 1), d2 = x - (lo + 2), d3 = x - (lo + 3);
  const double sixth = 1. / 6.;
  double r = d1 * d2 * d3 * -sixth * y[lo];
  r += d0 * d2 * d3 * 0.5 * y[lo + 1];
  r += d0 * d1 * d3 * -0.5 * y[lo + 2];
  r += d0 * d1 * d2 * sixth * y[lo + 3];
  return r;
}

typedef struct {
  int nDet, iDetCenter, nx, ny, geometry;
  double detInc, rotScale, xMin, xMax, yMin, yMax, xInc, yInc, fl, sdl;
} bp_ctx;

/* Backproject::Backproject (backprojectors.cpp:264-319) */
static void bp_setup(bp_ctx* c, const ora_geom* g, int nx, int ny, const double* roi) {
  c->detInc = g->detInc; c->nDet = g->nDet; c->iDetCenter = (g->nDet - 1) / 2;
  c->geometry = g->geometry;
  c->rotScale = g->geometry == ORA_GEOM_PARALLEL ? O_PI / g->nView : (2 * O_PI) / g->nView;
  c->nx = nx; c->ny = ny;
  double phmLen = g->viewDiameter / O_SQRT2;   /* include/projections.h:165 */
  c->xMin = -phmLen / 2; c->xMax = c->xMin + phmLen;
  c->yMin = -phmLen / 2; c->yMax = c->yMin + phmLen;
  if (roi) {
    if (roi[0] > c->xMin) c->xMin = roi[0];
    if (roi[2] < c->xMax) c->xMax = roi[2];
    if (roi[1] > c->yMin) c->yMin = roi[1];
    if (roi[3] < c->yMax) c->yMax = roi[3];
    if (c->xMin > c->xMax) { double t = c->xMin; c->xMin = c->xMax; c->xMax = t; }
    if (c->yMin > c->yMax) { double t = c->yMin; c->yMin = c->yMax; c->yMax = t; }
  }
  c->xInc = (c->xMax - c->xMin) / nx;
  c->yInc = (c->yMax - c->yMin) / ny;
  c->fl = g->focalLength; c->sdl = g->sourceDetectorLength;
}

/* value of one pixel for one view, table-family backprojectors
 * (Trig :365-404, Table :444-481, Equiangular :656-697, Equilinear :699-743) */
static double bp_table_value(const bp_ctx* c, int interp, const double* f, double theta,
                             double r, double phi) {
  int nDet = c->nDet;
  double pos, w = 1.0;
  if (c->geometry == ORA_GEOM_PARALLEL) {
    double L = r * cos(theta - phi);
    pos = L / c->detInc;
  } else {
    double da = theta - phi;
    double rc = r * cos(da), rs = r * sin(da);
    if (c->geometry == ORA_GEOM_EQUIANGULAR) {
      double flps = c->fl + rs;
      double gamma = atan(rc / flps);
      pos = gamma / c->detInc;
      w = flps * flps + (rc * rc);
    } else {
      double U = (c->fl + rs) / c->fl;
      double dp = rc / U;
      dp *= c->sdl / c->fl;
      pos = dp / c->detInc;
      w = U * U;
    }
  }
  double v = 0;
  if (interp == ORA_INTERP_NEAREST) {
    int i = c->iDetCenter + nearest_int(pos);
    if (i >= 0 && i < nDet) v = f[i];
    else return 0;
  } else if (interp == ORA_INTERP_LINEAR) {
    double pf = floor(pos);
    int i = c->iDetCenter + (int)pf;
    double fr = pos - pf;
    if (i >= 0 && i < nDet - 1) {
      if (c->geometry == ORA_GEOM_PARALLEL) v = (1 - fr) * f[i] + fr * f[i + 1];
      else v = f[i] + fr * (f[i + 1] - f[i]);
    } else return 0;
  } else {
    double p = c->iDetCenter + pos;
    if (p >= 0 && p < nDet) v = ora_cubic_interpolate(f, nDet, p);
    else return 0;
  }
  return c->geometry == ORA_GEOM_PARALLEL ? v : v / w;
}

int ora_backproject(const ora_geom* g, const double* filtered, int stride,
                    const double* angles, int iStart, int nViews, int nx, int ny,
                    const double* roi, int bproj, int interp, double* image, int postProcess,
                    int nThreads) {
  bp_ctx c;
  bp_setup(&c, g, nx, ny, roi);
  if (g->geometry != ORA_GEOM_PARALLEL) bproj = ORA_BP_TABLE;   /* :160-163 */
  int nDet = c.nDet;
  const int scaleShift = 32;
  const long scale = 1L << scaleShift, mask = scale - 1, half = scale / 2;
  const double invScale = 1. / scale;
  double x0 = c.xMin + c.xInc / 2, y0 = c.yMin + c.yInc / 2;
  double start_r = sqrt(x0 * x0 + y0 * y0), start_phi = atan2(y0, x0);   /* :491-502 */
#pragma omp parallel num_threads(nThreads > 0 ? nThreads : 1)
  {
    double* r = malloc((size_t)ny * sizeof(double));
    double* phi = malloc((size_t)ny * sizeof(double));
    double* delta = malloc((size_t)nDet * sizeof(double));
#pragma omp for schedule(dynamic, 4)
    for (int ix = 0; ix < nx; ix++) {
      double* col = &image[(size_t)ix * ny];
      /* the reference's accumulated pixel-centre coordinates (:422-428) */
      double x = x0;
      for (int k = 0; k < ix; k++) x += c.xInc;
      double y = y0;
      for (int iy = 0; iy < ny; iy++, y += c.yInc) {
        r[iy] = sqrt(x * x + y * y);
        phi[iy] = atan2(y, x);
      }
      for (int v = iStart; v < iStart + nViews; v++) {
        const double* f = &filtered[(size_t)(v - iStart) * stride];
        double theta = angles[v];
        if (bproj == ORA_BP_TRIG || bproj == ORA_BP_TABLE) {
          for (int iy = 0; iy < ny; iy++) {
            double val = bp_table_value(&c, interp, f, theta, r[iy], phi[iy]);
            col[iy] += bproj == ORA_BP_TRIG ? c.rotScale * val : val;
          }
        } else if (bproj == ORA_BP_DIFF) {   /* :517-570, column pointer drift kept */
          double ddx = c.xInc * cos(theta) / c.detInc, ddy = c.yInc * sin(theta) / c.detInc;
          double colStart = c.iDetCenter + start_r * cos(theta - start_phi) / c.detInc;
          for (int k = 0; k < ix; k++) colStart += ddx;
          if (interp == ORA_INTERP_LINEAR) {
            for (int i = 0; i < nDet - 1; i++) delta[i] = f[i + 1] - f[i];
            delta[nDet - 1] = 0;
          }
          double cur = colStart;
          double* p = col;
          for (int iy = 0; iy < ny; iy++, cur += ddy) {
            if (interp == ORA_INTERP_NEAREST) {
              int i = nearest_int(cur);
              if (i >= 0 && i < nDet) *p++ += f[i];
            } else if (interp == ORA_INTERP_LINEAR) {
              double pf = floor(cur);
              int i = (int)pf;
              double fr = cur - pf;
              if (i >= 0 && i <= nDet - 1) *p++ += f[i] + (fr * delta[i]);
            } else {
              if (cur >= 0 && cur < nDet) *p++ += ora_cubic_interpolate(f, nDet, cur);
            }
          }
        } else {   /* IntDiff, 32.32 fixed point (:579-653) */
          long ddx = nearest_long(c.xInc * cos(theta) / c.detInc * scale);
          long ddy = nearest_long(c.yInc * sin(theta) / c.detInc * scale);
          long colStart = nearest_long((start_r * cos(theta - start_phi) / c.detInc + c.iDetCenter) * scale);
          colStart += ddx * (long)ix;
          if (interp == ORA_INTERP_LINEAR) {
            for (int i = 0; i < nDet - 1; i++) delta[i] = (f[i + 1] - f[i]) * invScale;
            delta[nDet - 1] = 0;
          }
          long cur = colStart;
          for (int iy = 0; iy < ny; iy++, cur += ddy) {
            if (interp == ORA_INTERP_NEAREST) {
              int i = (int)((cur + half) >> scaleShift);
              if (i >= 0 && i <= nDet - 1) col[iy] += f[i];
            } else if (interp == ORA_INTERP_LINEAR) {
              long i = cur >> scaleShift;
              if (i >= 0 && i <= nDet - 1) col[iy] += f[i] + ((cur & mask) * delta[i]);
            } else {
              col[iy] += ora_cubic_interpolate(f, nDet, (double)cur / scale);
            }
          }
        }
      }
      if (postProcess && bproj != ORA_BP_TRIG)   /* ScaleImageByRotIncrement :330-336 */
        for (int iy = 0; iy < ny; iy++) col[iy] *= c.rotScale;
    }
    free(r); free(phi); free(delta);
  }
  return 1;
}

int ora_reconstruct(const ora_geom* g, const float* sino, const double* angles, int nx, int ny,
                    int filterId, double param, int method, int zeropad, int generation,
                    int bproj, int interp, double* image, int nThreads) {
  ora_procsig ps;   /* Reconstructor ctor: libctsim/reconstruct.cpp:50-103 */
  if (!ora_procsig_init(&ps, filterId, method, 1. / g->detInc, g->detInc, g->nDet, param,
                        generation, zeropad, 1, g->geometry, g->focalLength,
                        g->sourceDetectorLength))
    return 0;
  double* filt = malloc((size_t)g->nView * g->nDet * sizeof(double));
  ora_filter_views(&ps, sino, g->nView, filt, nThreads);
  memset(image, 0, (size_t)nx * ny * sizeof(double));
  ora_backproject(g, filt, g->nDet, angles, 0, g->nView, nx, ny, NULL, bproj, interp, image, 1,
                  nThreads);
  free(filt);
  ora_procsig_free(&ps);
  return 1;
}

/* ------------------------------------------------------------------------- */
/* Helical 180LI and half-scan feathering: libctsim/projections.cpp:231-439 */
/* (FP32 storage with FP64 weights, exactly as the reference)               */
/* ------------------------------------------------------------------------- */
/* fan angle of detector id: equiangular (projections.cpp:247, :378) uses the
 * integer centre (nDet-1)/2 times detInc; the equilinear restatement (no
 * reference counterpart) maps the same detector position through
 * atan(pos / SDL) (projections.cpp:1366-1370). */
static double det_gamma(const ora_geom* g, int id) {
  double pos = (id - (g->nDet - 1) / 2) * g->detInc;
  if (g->geometry == ORA_GEOM_EQUILINEAR) return atan(pos / g->sourceDetectorLength);
  return pos;
}

/* Projections::Helical180LI_Equiangular (projections.cpp:231-358); with
 * allowEquilinear, the same algorithm for an equilinear detector. */
int ora_helical180li_ex(const ora_geom* g, const float* in, int nView, int interpView,
                        float* out, double* outAngles, int* nViewOut, int allowEquilinear) {
  double dbeta = g->rotInc, fan = g->fanBeamAngle;
  int nDet = g->nDet, offsetView = 0;
  if (!(g->geometry == ORA_GEOM_EQUIANGULAR ||
        (allowEquilinear && g->geometry == ORA_GEOM_EQUILINEAR)))
    return 2;
  if (nView < (int)((2 * (O_PI + fan)) / dbeta) - 1) return 1;
  if (interpView < 0) interpView = (int)((O_PI + fan) / dbeta);
  else {
    if (interpView * dbeta < O_PI + fan || interpView * dbeta + O_PI + fan > nView * dbeta)
      return 1;
    offsetView = interpView - (int)((O_PI + fan) / dbeta);
  }
  int last = (int)((O_PI + fan) / dbeta);
  memset(out, 0, (size_t)(last + 1) * nDet * sizeof(float));
  for (int i = 0; i <= last; i++) outAngles[i] = (i + offsetView) * dbeta;
  int lastAcq = 2 * last;
  for (int iv = 0; iv <= lastAcq; iv++) {
    double beta = iv * dbeta;
    for (int id = 0; id < nDet; id++) {
      double gamma = det_gamma(g, id);
      int nv, nd;
      if (beta < O_PI + fan) { nd = id; nv = iv; }
      else {
        nd = -id + (nDet - 1);
        nv = nearest_int(((iv * dbeta) + 2 * gamma - O_PI) / dbeta);
      }
      if ((beta > fan - 2 * gamma) && (beta < 2 * O_PI + fan - 2 * gamma)) {
        float x = in[(size_t)(iv + offsetView) * nDet + id];
        float* o = &out[(size_t)nv * nDet + nd];
        if (beta > fan - 2 * gamma && beta <= 2 * fan)
          *o += (beta + 2 * gamma - fan) / (O_PI + 2 * gamma) * x;
        else if (beta > 2 * fan && beta <= O_PI - 2 * gamma)
          *o += (beta + 2 * gamma - fan) / (O_PI + 2 * gamma) * x;
        else if (beta > O_PI - 2 * gamma && beta <= O_PI + fan)
          *o += (beta + 2 * gamma - fan) / (O_PI + 2 * gamma) * x;
        else if (beta > O_PI + fan && beta <= O_PI + 2 * fan - 2 * gamma)
          *o += (2 * O_PI - beta - 2 * gamma + fan) / (O_PI - 2 * gamma) * x;
        else if (beta > O_PI + 2 * fan - 2 * gamma && beta <= 2 * O_PI)
          *o += (2 * O_PI - beta - 2 * gamma + fan) / (O_PI - 2 * gamma) * x;
        else if (beta > 2 * O_PI && beta <= 2 * O_PI + fan - 2 * gamma)
          *o += (2 * O_PI - beta - 2 * gamma + fan) / (O_PI - 2 * gamma) * x;
      }
    }
  }
  *nViewOut = last + 1;
  return 0;
}

int ora_helical180li(const ora_geom* g, const float* in, int nView, int interpView,
                     float* out, double* outAngles, int* nViewOut) {
  return ora_helical180li_ex(g, in, nView, interpView, out, outAngles, nViewOut, 0);
}

/* Projections::HalfScanFeather (projections.cpp:369-439).  The reference
 * takes gamma = (id - (nDet-1)/2) detInc for every fan geometry; with
 * trueGamma the equilinear detector's fan angle det_gamma() is used instead
 * (the restatement that goes with ora_helical180li_ex). */
int ora_halfscan_feather_ex(const ora_geom* g, float* data, int nView, int trueGamma) {
  double dbeta = g->rotInc, fan = g->fanBeamAngle;
  int nDet = g->nDet;
  if (nView != (int)((O_PI + fan) / dbeta) + 1) return 1;
  if (g->geometry == ORA_GEOM_PARALLEL) return 2;
  for (int iv2 = 0; iv2 < nView; iv2++) {
    double beta2 = iv2 * dbeta;
    for (int id2 = 0; id2 < nDet; id2++) {
      double gamma2 = trueGamma ? det_gamma(g, id2) : (id2 - (nDet - 1) / 2) * g->detInc;
      if (beta2 >= O_PI - 2 * gamma2) {
        int id1 = (nDet - 1) - id2;
        int iv1 = nearest_int(((iv2 * dbeta) + 2 * gamma2 - O_PI) / dbeta);
        float* d2 = &data[(size_t)iv2 * nDet + id2];
        float* d1 = &data[(size_t)iv1 * nDet + id1];
        *d1 = *d2;
        double x, beta1 = iv1 * dbeta, gamma1 = -gamma2;
        if (beta1 <= (fan - 2 * gamma1)) x = beta1 / (fan - 2 * gamma1);
        else if ((fan - 2 * gamma1 <= beta1) && beta1 <= O_PI - 2 * gamma1) x = 1;
        else if ((O_PI - 2 * gamma1 <= beta1) && (beta1 <= O_PI + fan))
          x = (O_PI + fan - beta1) / (fan + 2 * gamma1);
        else return 4;
        double w1 = (3 * x - 2 * x * x) * x, w2 = 1 - w1;
        *d1 *= w1;
        *d2 *= w2;
      }
    }
  }
  double sf = nView * g->rotInc / O_PI;
  for (size_t i = 0; i < (size_t)nView * nDet; i++) data[i] *= sf;
  return 0;
}

int ora_halfscan_feather(const ora_geom* g, float* data, int nView) {
  return ora_halfscan_feather_ex(g, data, nView, 0);
}

/* ------------------------------------------------------------------------- */
/* Projections::interpolateToParallel (projections.cpp:1250-1328) with      */
/* ParallelRaysums (:1339-1469) and LinearInterpolator (interpolator.h:187) */
/* ------------------------------------------------------------------------- */
typedef struct { double theta, t, raysum; } rb_coord;

static int rb_compare_t(const void* pa, const void* pb) {   /* compareByT */
  const rb_coord* a = pa;
  const rb_coord* b = pb;
  if (a->t == b->t) return a->theta < b->theta ? -1 : (a->theta > b->theta ? 1 : 0);
  return a->t < b->t ? -1 : 1;
}

static double normalize_angle(double th) {   /* mathfuncs.cpp:72-81 */
  while (th < 0.) th += O_TWOPI;
  while (th >= O_TWOPI) th -= O_TWOPI;
  return th;
}

/* LinearInterpolator::interpolate with x given, zero-outside off */
static double lin_interp(const double* x, const double* y, int n, double dX, int* lastFloor) {
  int iLower = -1, iUpper = n;
  if (lastFloor && *lastFloor >= 0 && x[*lastFloor] < dX) iLower = *lastFloor;
  while (iUpper - iLower > 1) {
    int iMiddle = (iUpper + iLower) >> 1;
    if (dX >= x[iMiddle]) iLower = iMiddle;
    else iUpper = iMiddle;
  }
  if (dX == x[0]) return y[0];
  if (dX < x[0]) return y[0];
  if (dX == x[n - 1]) return y[n - 1];
  if (dX > x[n - 1]) return y[n - 1];
  if (iLower < 0 || iLower >= n) return 0;
  if (lastFloor) *lastFloor = iLower;
  return y[iLower] + (y[iUpper] - y[iLower]) * ((dX - x[iLower]) / (x[iUpper] - x[iLower]));
}

int ora_interpolate_to_parallel(const ora_geom* g, double rotStart, double detStart,
                                const float* in, const double* viewAngles, float* out,
                                double* outAngles, double* outHdr) {
  int nDet = g->nDet, nView = g->nView;
  if (g->geometry == ORA_GEOM_PARALLEL) return 1;
  double rotInc = O_TWOPI / nView;
  double dStart = -g->viewDiameter / 2, dInc = g->viewDiameter / nDet;
  if (nDet % 2 == 0) dInc = g->viewDiameter / (nDet - 1);
  rb_coord* c = malloc((size_t)nView * nDet * sizeof(rb_coord));
  for (int v = 0; v < nView; v++) {
    double detPos = detStart;
    for (int d = 0; d < nDet; d++) {
      rb_coord* pc = &c[(size_t)v * nDet + d];
      if (g->geometry == ORA_GEOM_EQUILINEAR) {
        double fan = atan(detPos / g->sourceDetectorLength);
        pc->theta = viewAngles[v] + fan;
        pc->t = g->focalLength * sin(fan);
      } else {
        pc->theta = viewAngles[v] + detPos;
        pc->t = g->focalLength * sin(detPos);
      }
      pc->theta = normalize_angle(pc->theta);
      pc->raysum = in[(size_t)v * nDet + d];
      detPos += g->detInc;
    }
  }
  qsort(c, (size_t)nView * nDet, sizeof(rb_coord), rb_compare_t);
  double* th = malloc(nView * sizeof(double));
  double* rs = malloc(nView * sizeof(double));
  for (int iD = 0; iD < nDet; iD++) {
    for (int i = 0; i < nView; i++) {
      th[i] = c[(size_t)iD * nView + i].theta;
      rs[i] = c[(size_t)iD * nView + i].raysum;
    }
    double a = rotStart;
    int last = -1;
    for (int iV = 0; iV < nView; iV++, a += rotInc)
      out[(size_t)iV * nDet + iD] = (float)lin_interp(th, rs, nView, a, &last);
  }
  double* dp = malloc(nDet * sizeof(double));
  double* row = malloc(nDet * sizeof(double));
  for (int i = 0; i < nDet; i++) dp[i] = c[(size_t)i * nView].t;
  double a = rotStart;
  for (int iV = 0; iV < nView; iV++, a += rotInc) {
    outAngles[iV] = a;
    for (int i = 0; i < nDet; i++) row[i] = out[(size_t)iV * nDet + i];
    double pos = dStart;
    int last = -1;
    for (int iD = 0; iD < nDet; iD++, pos += dInc)
      out[(size_t)iV * nDet + iD] = (float)lin_interp(dp, row, nDet, pos, &last);
  }
  outHdr[0] = rotInc;
  outHdr[1] = dStart;
  outHdr[2] = dInc;
  free(c); free(th); free(rs); free(dp); free(row);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Rasteriser: Phantom::convertToImagefile (phantom.cpp:462-542) with        */
/* PhantomElement::isPointInside (phantom.cpp:913-976)                      */
/* ------------------------------------------------------------------------- */
static int point_inside(const ora_pelem* e, double x, double y) {
  m_apply(e->phm2obj, &x, &y);
  switch (e->type) {
    case ORA_PELEM_RECTANGLE: return !(x > 1. || x < -1. || y > 1. || y < -1.);
    case ORA_PELEM_TRIANGLE: return !(y < 0. || y > 1. - x || y > 1. + x);
    case ORA_PELEM_ELLIPSE:
      if (x > 1. || x < -1. || y > 1. || y < -1.) return 0;
      return !(x * x + y * y > 1.);
    case ORA_PELEM_SEGMENT:
      if (x > 1. || x < -1. || y > 0.) return 0;
      x *= e->u; y *= e->v;
      return !(x * x + (y - e->v) * (y - e->v) > e->u * e->u + e->v * e->v);
    case ORA_PELEM_SECTOR:
      if (x > 1. || x < -1. || y > 1.) return 0;
      if (y > 1. - x || y > 1. + x) return 0;
      x *= e->u; y *= e->v;
      return !(x * x + (y - e->v) * (y - e->v) > e->u * e->u + e->v * e->v);
    default: return 0;
  }
}

void ora_phantom_to_image(const ora_phantom* p, int nx, int ny, double viewRatio, int nsample,
                          double* image, double extent[4], int nThreads) {
  if (nsample < 1) nsample = 1;
  double dx = p->xmax - p->xmin, dy = p->ymax - p->ymin;
  double xc = p->xmin + dx / 2, yc = p->ymin + dy / 2;
  double maxAxis = dx > dy ? dx : dy;
  double half = viewRatio * (O_SQRT2 * maxAxis / O_SQRT2 / 2);
  double xmin = xc - half, xmax = xc + half, ymin = yc - half, ymax = yc + half;
  double xinc = (xmax - xmin) / nx, yinc = (ymax - ymin) / ny;
  double kxinc = xinc / nsample, kyinc = yinc / nsample, kxofs = kxinc / 2, kyofs = kyinc / 2;
  if (extent) { extent[0] = xmin; extent[1] = xmax; extent[2] = ymin; extent[3] = ymax; }
  memset(image, 0, (size_t)nx * ny * sizeof(double));
#pragma omp parallel for schedule(dynamic, 4) num_threads(nThreads > 0 ? nThreads : 1)
  for (int ix = 0; ix < nx; ix++) {
    double x = xmin;
    for (int k = 0; k < ix; k++) x += xinc;
    for (int k = 0; k < p->n; k++) {
      const ora_pelem* e = &p->e[k];
      double y = ymin;
      for (int iy = 0; iy < ny; iy++, y += yinc) {
        double a = 0, xi = x + kxofs;
        for (int kx = 0; kx < nsample; kx++, xi += kxinc) {
          double yi = y + kyofs;
          for (int ky = 0; ky < nsample; ky++, yi += kyinc)
            if (point_inside(e, xi, yi)) a += e->atten;
        }
        image[(size_t)ix * ny + iy] += a;
      }
    }
    if (nsample > 1) {
      double f = 1.0 / (double)(nsample * nsample);
      for (int iy = 0; iy < ny; iy++) image[(size_t)ix * ny + iy] *= f;
    }
  }
}

/* Pixel-image projector: the exact transpose of the parallel-beam table
 * backprojector with linear interpolation (backprojectors.cpp:444-481),
 * without the final rotScale.  sino[v][d] = sum over pixels of
 * image * (linear weight of that pixel's detector position on d). */
int ora_project_image(const ora_geom* g, const double* image, int nx, int ny,
                      const double* angles, int nView, double* sino, int nThreads) {
  bp_ctx c;
  bp_setup(&c, g, nx, ny, NULL);
  int nDet = c.nDet;
  memset(sino, 0, (size_t)nView * nDet * sizeof(double));
#pragma omp parallel for schedule(dynamic, 4) num_threads(nThreads > 0 ? nThreads : 1)
  for (int v = 0; v < nView; v++) {
    double th = angles[v];
    double* row = &sino[(size_t)v * nDet];
    double x = c.xMin + c.xInc / 2;
    for (int ix = 0; ix < nx; ix++, x += c.xInc) {
      double y = c.yMin + c.yInc / 2;
      for (int iy = 0; iy < ny; iy++, y += c.yInc) {
        double r = sqrt(x * x + y * y), phi = atan2(y, x);
        double pos = r * cos(th - phi) / c.detInc;
        double pf = floor(pos);
        int i = c.iDetCenter + (int)pf;
        double fr = pos - pf, val = image[(size_t)ix * ny + iy];
        if (i >= 0 && i < nDet - 1) {
          row[i] += (1 - fr) * val;
          row[i + 1] += fr * val;
        }
      }
    }
  }
  return 1;
}

/* ---- ImageFile::comparativeStatistics (libctsim/imagefile.cpp:186-240) ----
 * FP32 images [nx][ny] (column-major, v[ix][iy]); the differences and the
 * 2x2 block sums are FP32 expressions there, the sums FP64, in this order. */
int ora_image_compare(const float* a, const float* b, int nx, int ny, double out[3]) {
  if (nx <= 0 || ny <= 0) return 0;
  double mean = 0.;
  for (int ix = 0; ix < nx; ix++)
    for (int iy = 0; iy < ny; iy++) mean += a[(size_t)ix * ny + iy];
  mean /= (unsigned int)nx * (unsigned int)ny;
  double sqErr = 0., absErr = 0., sqDev = 0., absVal = 0.;
  for (int ix = 0; ix < nx; ix++)
    for (int iy = 0; iy < ny; iy++) {
      const size_t i = (size_t)ix * ny + iy;
      const float fd = a[i] - b[i];
      const double diff = fd;
      sqErr += diff * diff;
      absErr += fabs(diff);
      const double dm = a[i] - mean;
      sqDev += dm * dm;
      absVal += fabs((double)a[i]);
    }
  out[0] = sqrt(sqErr / sqDev);
  out[1] = absErr / absVal;
  const int hx = nx / 2, hy = ny / 2;
  double eMax = -1;
  for (int i3 = 0; i3 < hx; i3++)
    for (int iy = 0; iy < hy; iy++) {
      const size_t o0 = (size_t)(2 * i3) * ny + 2 * iy, o1 = o0 + ny;
      const float sa = a[o0] + a[o1] + a[o0 + 1] + a[o1 + 1];
      const float sb = b[o0] + b[o1] + b[o0 + 1] + b[o1 + 1];
      const double err = fabs(0.25 * sa - 0.25 * sb);
      if (err > eMax) eMax = err;
    }
  out[2] = eMax;
  return 1;
}

/* ------------------------------------------------------------------------- */
/* Polar and direct-Fourier images: Projections::convertPolar /             */
/* convertFFTPolar (projections.cpp:953-1180) and the Fourier               */
/* reconstruction of the GUI (src/views.cpp:2828-2849): convertFFTPolar,    */
/* ImageFile::ifft (imagefile.cpp:770-826), magnitude (:1175-1198) and      */
/* Fourier::shuffleFourierToNaturalOrder (fourier.cpp:31-63).  FFTW's       */
/* transforms are restated as DFTs (radix-2 for powers of two).             */
/* ------------------------------------------------------------------------- */

/* Fourier::shuffleFourierToNaturalOrder: new[d] = old[nat_src(n, d)] */
static int nat_src(int n, int d) {
  if (n % 2) {
    const int h = (n - 1) / 2;
    return d == h ? 0 : (d > h ? d - h : d + h + 1);
  }
  const int h = n / 2;
  return d == h ? 0 : (d < h ? d + h : d - h);
}
/* Fourier::shuffleNaturalToFourierOrder: new[d] = old[fou_src(n, d)] */
static int fou_src(int n, int d) {
  if (n % 2) {
    const int h = (n - 1) / 2;
    return d == 0 ? h : (d <= h ? d + h : d - h - 1);
  }
  const int h = n / 2;
  return d == 0 ? h : (d < h ? d + h : d - h);
}

/* DFT of n complex values (re, im) in place; sign -1 forward (FFTW_FORWARD),
   +1 backward; unnormalised */
static void dft_inplace(double* re, double* im, int n, int sign) {
  if (n <= 1) return;
  if ((n & (n - 1)) == 0) {   /* iterative radix-2 Cooley-Tukey */
    for (int i = 1, j = 0; i < n; i++) {
      int bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) {
        double t = re[i]; re[i] = re[j]; re[j] = t;
        t = im[i]; im[i] = im[j]; im[j] = t;
      }
    }
    for (int len = 2; len <= n; len <<= 1) {
      for (int k = 0; k < len / 2; k++) {
        const double a = sign * O_TWOPI * k / len, wr = cos(a), wi = sin(a);
        for (int i = 0; i < n; i += len) {
          const int u = i + k, v = i + k + len / 2;
          const double xr = re[v] * wr - im[v] * wi, xi = re[v] * wi + im[v] * wr;
          re[v] = re[u] - xr; im[v] = im[u] - xi;
          re[u] += xr; im[u] += xi;
        }
      }
    }
    return;
  }
  double* tr = malloc(sizeof(double) * n);
  double* ti = malloc(sizeof(double) * n);
  for (int k = 0; k < n; k++) {
    double sr = 0, si = 0;
    for (int j = 0; j < n; j++) {
      const double a = sign * O_TWOPI * (double)(((long long)j * k) % n) / n;
      const double c = cos(a), s = sin(a);
      sr += re[j] * c - im[j] * s;
      si += re[j] * s + im[j] * c;
    }
    tr[k] = sr; ti[k] = si;
  }
  memcpy(re, tr, sizeof(double) * n);
  memcpy(im, ti, sizeof(double) * n);
  free(tr); free(ti);
}

/* Projections::calcArrayPolarCoordinates (projections.cpp:1113-1149) */
static void polar_coords(int nx, int ny, double viewDiameter, double rotInc, double rotStart,
                         int nDetWithZeros, double zeropadRatio, double detInc, double* pView,
                         double* pDet) {
  double xMin = -viewDiameter / 2, xMax = xMin + viewDiameter;
  double yMin = -viewDiameter / 2, yMax = yMin + viewDiameter;
  const double xCent = (xMin + xMax) / 2, yCent = (yMin + yMax) / 2;
  xMin = (xMin - xCent) * zeropadRatio + xCent;
  xMax = (xMax - xCent) * zeropadRatio + xCent;
  yMin = (yMin - yCent) * zeropadRatio + yCent;
  yMax = (yMax - yCent) * zeropadRatio + yCent;
  const double xInc = (xMax - xMin) / nx, yInc = (yMax - yMin) / ny;
  const double detCenter = (nDetWithZeros - 1) / 2.;
  double x = xMin + xInc / 2;
  for (int ix = 0; ix < nx; x += xInc, ix++) {
    double y = yMin + yInc / 2;
    for (int iy = 0; iy < ny; y += yInc, iy++) {
      double r = sqrt(x * x + y * y);
      double phi = atan2(y, x);
      if (phi <= -rotInc / 2) phi += O_TWOPI;
      if (phi >= O_PI - (rotInc / 2)) {
        phi -= O_PI;
        r = -r;
      }
      pView[(size_t)ix * ny + iy] = (phi - rotStart) / rotInc;
      pDet[(size_t)ix * ny + iy] = (r / detInc) + detCenter;
    }
  }
}

/* BilinearPolarInterpolator::interpolate (include/interpolator.h:110-154) of
   one component of m [nAngle][nPos] */
static double bilinear_polar(const double* m, int nAngle, int nPos, double dAngle, double dPos) {
#define M(a, p) m[(size_t)(a) * nPos + (p)]
  const int fa0 = (int)floor(dAngle), fp0 = (int)floor(dPos);
  const double fa = dAngle - fa0, fp = dPos - fp0;
  if (fa0 < -1 || fp0 < 0 || fa0 > nAngle - 1 || fp0 > nPos - 1) return 0;
  if (fa0 == -1 && fp0 == nPos - 1) return M(0, nPos - 1) + fa * (M(nAngle - 1, fp0) - M(0, fp0));
  if (fa0 == nAngle - 1 && fp0 == nPos - 1)
    return M(nAngle - 1, nPos - 1) + fa * (M(0, fp0) - M(nAngle - 1, fp0));
  if (fp0 == nPos - 1) return M(fa0, fp0) + fa * (M(fa0 + 1, fp0) - M(fa0, fp0));
  if (fa0 == nAngle - 1) {
    const int lo = (nPos - 1) - fp0, up = (nPos - 1) - (fp0 + 1);
    return (1 - fa) * (1 - fp) * M(fa0, fp0) + fa * (1 - fp) * M(0, lo) +
           fp * (1 - fa) * M(fa0, fp0 + 1) + fa * fp * M(0, up);
  }
  if (fa0 == -1) {
    const int lo = (nPos - 1) - fp0, up = (nPos - 1) - (fp0 + 1);
    return (1 - fa) * (1 - fp) * M(nAngle - 1, lo) + fa * (1 - fp) * M(fa0 + 1, fp0) +
           fp * (1 - fa) * M(nAngle - 1, up) + fa * fp * M(fa0 + 1, fp0 + 1);
  }
  return (1 - fa) * (1 - fp) * M(fa0, fp0) + fa * (1 - fp) * M(fa0 + 1, fp0) +
         fp * (1 - fa) * M(fa0, fp0 + 1) + fa * fp * M(fa0 + 1, fp0 + 1);
#undef M
}

/* Projections::interpolatePolar (projections.cpp:1136-1180); its loops run ix
   over ny as well (:1151), so only columns ix < min(nx, ny) are written */
static void polar_interp(const double* re, const double* im, int nView, int nPos,
                         const double* pView, const double* pDet, int nx, int ny, int interp,
                         float* outRe, float* outIm) {
  const int cols = nx < ny ? nx : ny;
  for (int ix = 0; ix < cols; ix++)
    for (int iy = 0; iy < ny; iy++) {
      const size_t i = (size_t)ix * ny + iy;
      double vr = 0, vi = 0;
      if (interp == 0) {
        const double a = pView[i], p = pDet[i];
        unsigned int iv = (unsigned int)(a > 0 ? (int)(a + 0.5) : (int)(a - 0.5));
        const unsigned int id = (unsigned int)(p > 0 ? (int)(p + 0.5) : (int)(p - 0.5));
        if (iv == (unsigned int)nView) iv = 0;
        if (id < (unsigned int)nPos && iv < (unsigned int)nView) {
          vr = re[(size_t)iv * nPos + id];
          vi = im ? im[(size_t)iv * nPos + id] : 0;
        }
      } else {
        vr = bilinear_polar(re, nView, nPos, pView[i], pDet[i]);
        vi = im ? bilinear_polar(im, nView, nPos, pView[i], pDet[i]) : 0;
      }
      outRe[i] = (float)vr;
      if (outIm) outIm[i] = (float)vi;
    }
}

/* the parallel projections the polar conversions start from: the input, or
   interpolateToParallel of fan-beam data (rotStart 0 afterwards) */
static float* polar_source(const ora_geom* g, double rotStart, double detStart, const float* sino,
                           const double* angles, double* rs, double* ri, double* di) {
  float* p = malloc(sizeof(float) * (size_t)g->nView * g->nDet);
  if (g->geometry == ORA_GEOM_PARALLEL) {
    memcpy(p, sino, sizeof(float) * (size_t)g->nView * g->nDet);
    *rs = rotStart; *ri = g->rotInc; *di = g->detInc;
  } else {
    double* oa = malloc(sizeof(double) * g->nView);
    double hdr[3];
    ora_interpolate_to_parallel(g, rotStart, detStart, sino, angles, p, oa, hdr);
    free(oa);
    *rs = 0; *ri = hdr[0]; *di = hdr[2];
  }
  return p;
}

int ora_convert_polar(const ora_geom* g, double rotStart, double detStart, const float* sino,
                      const double* angles, int nx, int ny, int interp, float* out) {
  double rs, ri, di;
  float* p = polar_source(g, rotStart, detStart, sino, angles, &rs, &ri, &di);
  const size_t n = (size_t)g->nView * g->nDet;
  double* re = malloc(sizeof(double) * n);
  for (size_t i = 0; i < n; i++) re[i] = p[i];
  double* pv = malloc(sizeof(double) * (size_t)nx * ny);
  double* pd = malloc(sizeof(double) * (size_t)nx * ny);
  polar_coords(nx, ny, g->viewDiameter, ri, rs, g->nDet, 1., di, pv, pd);
  memset(out, 0, sizeof(float) * (size_t)nx * ny);
  polar_interp(re, NULL, g->nView, g->nDet, pv, pd, nx, ny, interp, out, NULL);
  free(p); free(re); free(pv); free(pd);
  return 0;
}

/* ProcessSignal::addZeropadFactor (procsignal.cpp:867-881) */
int ora_add_zeropad_factor(int n, int zeropad) {
  if (zeropad > 0) {
    const double lb = log(n) / log(2);
    return 1 << ((int)floor(lb) + zeropad);
  }
  return n;
}

int ora_convert_fft_polar(const ora_geom* g, double rotStart, double detStart, const float* sino,
                          const double* angles, int nx, int ny, int interp, int zeropad,
                          float* outRe, float* outIm) {
  double rs, ri, di;
  float* p = polar_source(g, rotStart, detStart, sino, angles, &rs, &ri, &di);
  const int nDet = g->nDet, nView = g->nView;
  const int nInterp = (int)(double)sqrt((double)(unsigned int)(nx * nx + ny * ny));
  const int N = ora_add_zeropad_factor(nInterp, zeropad);
  const double projScale = nInterp / (g->viewDiameter * 0.05);
  const double zpRatio = (double)N / (double)nInterp;
  const double interpScale = nDet / (double)nInterp;
  const double fftScale = 1. / (double)(nInterp * nInterp);
  const int iMid = nInterp / 2;
  const double dMid = nInterp / 2.;
  const int zeros = N - nInterp;
  double* re = malloc(sizeof(double) * (size_t)nView * N);
  double* im = malloc(sizeof(double) * (size_t)nView * N);
  double* vr = malloc(sizeof(double) * (N > nInterp ? N : nInterp));
  double* vi = malloc(sizeof(double) * (N > nInterp ? N : nInterp));
  double* tr = malloc(sizeof(double) * (N > nInterp ? N : nInterp));
  for (int v = 0; v < nView; v++) {
    const float* y = p + (size_t)v * nDet;
    for (int i = 0; i < nInterp; i++) {   /* LinearInterpolator<float>, zero outside */
      const double x = (nDet / 2.) + (i - dMid) * interpScale;
      double r;
      if (x == 0) r = y[0];
      else if (x < 0) r = 0;
      else if (x == nDet - 1) r = y[nDet - 1];
      else if (x > nDet - 1) r = 0;
      else {
        const int f = (int)floor(x);
        r = y[f] + (y[f + 1] - y[f]) * (x - f);
      }
      vr[i] = r * projScale;
      vi[i] = 0;
    }
    for (int d = 0; d < nInterp; d++) tr[d] = vr[nat_src(nInterp, d)];
    memcpy(vr, tr, sizeof(double) * nInterp);
    if (zeros > 0) {
      for (int i = nInterp - 1; i >= iMid; i--) { vr[i + zeros] = vr[i]; vi[i + zeros] = vi[i]; }
      for (int i = iMid; i < iMid + zeros; i++) vr[i] = vi[i] = 0;
    }
    dft_inplace(vr, vi, N, -1);
    for (int d = 0; d < N; d++) {
      re[(size_t)v * N + d] = vr[nat_src(N, d)] * fftScale;
      im[(size_t)v * N + d] = vi[nat_src(N, d)] * fftScale;
    }
  }
  double* pv = malloc(sizeof(double) * (size_t)nx * ny);
  double* pd = malloc(sizeof(double) * (size_t)nx * ny);
  polar_coords(nx, ny, g->viewDiameter, ri, rs, N, zpRatio, di * interpScale, pv, pd);
  memset(outRe, 0, sizeof(float) * (size_t)nx * ny);
  memset(outIm, 0, sizeof(float) * (size_t)nx * ny);
  polar_interp(re, im, nView, N, pv, pd, nx, ny, interp, outRe, outIm);
  free(p); free(re); free(im); free(vr); free(vi); free(tr); free(pv); free(pd);
  return N;
}

/* ImageFile::ifft + magnitude + Fourier::shuffleFourierToNaturalOrder of a
   complex FP32 image [nx][ny] -> out (FP32) */
void ora_ifft_magnitude(const float* inRe, const float* inIm, int nx, int ny, float* out) {
  const size_t n = (size_t)nx * ny;
  double* re = malloc(sizeof(double) * n);
  double* im = malloc(sizeof(double) * n);
  /* shuffleNaturalToFourierOrder (fourier.cpp:66-98): each column, then each row */
  for (int ix = 0; ix < nx; ix++)
    for (int iy = 0; iy < ny; iy++) {
      const size_t s = (size_t)fou_src(nx, ix) * ny + fou_src(ny, iy);
      re[(size_t)ix * ny + iy] = inRe[s];
      im[(size_t)ix * ny + iy] = inIm[s];
    }
  /* FFTW_BACKWARD 2-D DFT, unnormalised: along iy, then along ix */
  double* cr = malloc(sizeof(double) * (nx > ny ? nx : ny));
  double* ci = malloc(sizeof(double) * (nx > ny ? nx : ny));
  for (int ix = 0; ix < nx; ix++) dft_inplace(re + (size_t)ix * ny, im + (size_t)ix * ny, ny, 1);
  for (int iy = 0; iy < ny; iy++) {
    for (int ix = 0; ix < nx; ix++) { cr[ix] = re[(size_t)ix * ny + iy]; ci[ix] = im[(size_t)ix * ny + iy]; }
    dft_inplace(cr, ci, nx, 1);
    for (int ix = 0; ix < nx; ix++) { re[(size_t)ix * ny + iy] = cr[ix]; im[(size_t)ix * ny + iy] = ci[ix]; }
  }
  /* FP32 image, magnitude in FP32 (imagefile.cpp:1189), natural order */
  float* mag = malloc(sizeof(float) * n);
  for (size_t i = 0; i < n; i++) {
    const float r = (float)re[i], m = (float)im[i];
    mag[i] = sqrtf(r * r + m * m);
  }
  for (int ix = 0; ix < nx; ix++)
    for (int iy = 0; iy < ny; iy++)
      out[(size_t)ix * ny + iy] = mag[(size_t)nat_src(nx, ix) * ny + nat_src(ny, iy)];
  free(re); free(im); free(cr); free(ci); free(mag);
}
