// swe_dual.cuh -- forward-mode dual numbers and the step's point-wise
// functions templated on the scalar type, for the discrete adjoint.
//
// Dual<N> carries a value and N partial derivatives.  Every templated function
// below repeats the operation order of its double counterpart in
// swe_physics.cuh, so the value part of a Dual evaluation is bit-identical to
// the forward step and every branch (dry clamps, limiter, min/max selections,
// wet/dry thresholds) is taken exactly as in the forward pass; derivatives are
// those of the branch taken; derivative parts use explicit fused
// multiply-adds (values never do).  Derivatives of sqrt at 0 are taken as 0: a zero
// depth only reaches sqrt from a dry-clamped interface value, which is
// locally constant.
#pragma once

#include "swe_physics.cuh"

namespace swe {

template <int N>
struct Dual {
  double v;
  double d[N];
  SWE_HD Dual() : v(0.) {
    for (int k = 0; k < N; ++k) d[k] = 0.;
  }
  SWE_HD Dual(double x) : v(x) {
    for (int k = 0; k < N; ++k) d[k] = 0.;
  }
  SWE_HD static Dual var(double x, int k) {
    Dual r(x);
    r.d[k] = 1.;
    return r;
  }
};

SWE_HD double val(double x) { return x; }
template <int N>
SWE_HD double val(const Dual<N>& x) {
  return x.v;
}

template <int N>
SWE_HD Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v + b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int N>
SWE_HD Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v - b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int N>
SWE_HD Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r(-a.v);
  for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int N>
SWE_HD Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v * b.v);
  for (int k = 0; k < N; ++k) r.d[k] = fma(a.d[k], b.v, a.v * b.d[k]);
  return r;
}
template <int N>
SWE_HD Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  const double q = SWE_DIV(a.v, b.v);  // the value keeps the exact quotient
  Dual<N> r(q);
  const double ib = SWE_DIV(1., b.v);
  for (int k = 0; k < N; ++k) r.d[k] = fma(-q, b.d[k], a.d[k]) * ib;
  return r;
}
template <int N>
SWE_HD Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N>
SWE_HD Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N>
SWE_HD Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N>
SWE_HD Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N>
SWE_HD Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r(a.v * b);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b;
  return r;
}
template <int N>
SWE_HD Dual<N> operator*(double a, const Dual<N>& b) {
  Dual<N> r(a * b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a * b.d[k];
  return r;
}
template <int N>
SWE_HD Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N>
SWE_HD Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }

SWE_HD double tsqrt(double x) { return SWE_SQRT(x); }
template <int N>
SWE_HD Dual<N> tsqrt(const Dual<N>& a) {
  const double s = SWE_SQRT(a.v);
  Dual<N> r(s);
  const double g = (s > 0.) ? SWE_DIV(0.5, s) : 0.;
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * g;
  return r;
}
SWE_HD double tfabs(double x) { return fabs(x); }
template <int N>
SWE_HD Dual<N> tfabs(const Dual<N>& a) {
  return signbit(a.v) ? -a : a;
}
// std::min / std::max semantics on the values
template <class T>
SWE_HD T tmin(const T& a, const T& b) {
  return dlt(val(b), val(a)) ? b : a;
}
template <class T>
SWE_HD T tmax(const T& a, const T& b) {
  return dlt(val(a), val(b)) ? b : a;
}

// ---------------------------------------------------------- templated physics
// src/Assigners.cpp:8-20
template <class T>
SWE_HD void prim_assign_t(const T& b, const T& w, T u, T v, T* ow, T* ou, T* ov) {
  T h = w - b;
  if (!is_wet(val(h))) {
    *ow = b;
    *ou = T(0.);
    *ov = T(0.);
    return;
  }
  if (dltc(val(h), kEta1)) {
    T s = (kSqrt2 * h) / tsqrt(h * h + kEta2);
    u = u * s;
    v = v * s;
  }
  *ow = w;
  *ou = u;
  *ov = v;
}

// include/SpaceDisc.h:4-18
template <class T>
SWE_HD void elem_flux_t(double nx, double ny, const T& h, const T& hu, const T& hv, T* f) {
  f[0] = T(0.);
  f[1] = T(0.);
  f[2] = T(0.);
  if (is_wet(val(h))) {
    T hveln = hu * nx + hv * ny;
    f[0] = hveln;
    T q = hveln / h;
    f[1] = q * hu + (0.5 * h * h) * nx;
    f[2] = q * hv + (0.5 * h * h) * ny;
  }
}

// src/Fluxes.cpp:5-26
template <class T>
SWE_HD void wavespeeds_t(int ws, const T& ul, const T& hl, const T& ur, const T& hr, T* a0, T* a1) {
  T cl = tsqrt(hl), cr = tsqrt(hr);
  if (ws == 0) {
    T ap = tmax(tfabs(ul) + cl, tfabs(ur) + cr);
    *a0 = -ap;
    *a1 = ap;
  } else if (ws == 1) {
    *a0 = tmin(ul - cl, ur - cr);
    *a1 = tmax(ul + cl, ur + cr);
  } else {
    T uRoe = (cl * ul + cl * ur) / (cl + cr);
    T cRoe = tsqrt(0.5 * (hl + hr));
    *a0 = tmin(ul - cl, uRoe - cRoe);
    *a1 = tmax(ur + cr, uRoe + cRoe);
  }
}

// include/Fluxes.h:14-111 for interface states (wl, ul, vl), (wr, ur, vr)
// over an edge with normal n, tangent t and bathymetry b (all of which are
// values of type T except the 2-D geometry).
template <class T>
SWE_HD void flux_t(int flux, int ws, double nx, double ny, double tx, double ty, const T& b, const T& Lw,
                   const T& Lu, const T& Lv, const T& Rw, const T& Ru, const T& Rv, T* F) {
  F[0] = T(0.);
  F[1] = T(0.);
  F[2] = T(0.);
  T ul = Lu * nx + Lv * ny;
  T hl = Lw - b;
  T ur = Ru * nx + Rv * ny;
  T hr = Rw - b;
  if (!dgtc(val(hl + hr), kMinCapture)) return;
  if (flux == 0) {
    T a0, a1;
    wavespeeds_t(ws, ul, hl, ur, hr, &a0, &a1);
    T al = tmin(T(0.), a0);
    T ar = tmax(T(0.), a1);
    if (!dgtc(val(ar - al), kMinCapture)) return;
    T Ul[3] = {hl, hl * Lu, hl * Lv};
    T Ur[3] = {hr, hr * Ru, hr * Rv};
    T Fl[3], Fr[3];
    elem_flux_t(nx, ny, Ul[0], Ul[1], Ul[2], Fl);
    elem_flux_t(nx, ny, Ur[0], Ur[1], Ur[2], Fr);
    for (int q = 0; q < 3; ++q) F[q] = (ar * Fl[q] - al * Fr[q] + (al * ar) * (Ur[q] - Ul[q])) / (ar - al);
    return;
  }
  T vl = Lu * tx + Lv * ty;
  T vr = Ru * tx + Rv * ty;
  T al, ar;
  wavespeeds_t(ws, ul, hl, ur, hr, &al, &ar);
  T ustar = (ar - ur) * hr * ur - (al - ul) * hl * ul + 0.5 * (hl * hl - hr * hr);
  ustar = ustar / (hr * (ar - ur) - hl * (al - ul));
  if (!dgt0(val(ustar))) {
    T Ur[3] = {hr, hr * Ru, hr * Rv};
    T us = vr * tx + ustar * ty;
    T vs = vr * nx + ustar * ny;
    T hs = hr * (ar - ur) / (ar - ustar);
    T Us[3] = {hs, hs * us, hs * vs};
    T Fr[3];
    elem_flux_t(nx, ny, Ur[0], Ur[1], Ur[2], Fr);
    T s = tmax(T(0.), ar);
    for (int q = 0; q < 3; ++q) F[q] = Fr[q] + s * (Us[q] - Ur[q]);
  } else {
    T Ul[3] = {hl, hl * Lu, hl * Lv};
    T us = vl * tx + ustar * ty;
    T vs = vl * nx + ustar * ny;
    T hs = hl * (al - ul) / (al - ustar);
    T Us[3] = {hs, hs * us, hs * vs};
    T Fl[3];
    elem_flux_t(nx, ny, Ul[0], Ul[1], Ul[2], Fl);
    T s = tmin(T(0.), al);
    for (int q = 0; q < 3; ++q) F[q] = Fl[q] + s * (Us[q] - Ul[q]);
  }
}

// src/PointOperations.cpp:42-48, templated
template <class T>
SWE_HD void plane_gradient_t(const T& p0x, const T& p0y, const T& p0z, const T& p1x, const T& p1y, const T& p1z,
                             const T& p2x, const T& p2y, const T& p2z, T* gx, T* gy) {
  T a00 = p1x - p0x, a01 = p1y - p0y, b0 = p1z - p0z;
  T a10 = p2x - p0x, a11 = p2y - p0y, b1 = p2z - p0z;
  if (dlt(fabs(val(a00)), fabs(val(a10)))) {
    T t;
    t = a00; a00 = a10; a10 = t;
    t = a01; a01 = a11; a11 = t;
    t = b0; b0 = b1; b1 = t;
  }
  T l10 = a10;
  if (val(a00) != 0.) l10 = a10 / a00;
  T u11 = a11 - l10 * a01;
  T y1 = b1 - l10 * b0;
  T x1 = y1 / u11;
  T x0 = (b0 - a01 * x1) / a00;
  *gx = x0;
  *gy = x1;
}

// Root x of x^3 + b x^2 + c x + d found by the reference's bisection
// (src/PointOperations.cpp:26-40); derivatives by the implicit-function
// theorem at the root (dx = -(dd + dc x + db x^2) / f'(x)), or zero when the
// bisection returned an end point.
template <int N>
SWE_HD Dual<N> bisection_t(const Dual<N>& d, const Dual<N>& c, const Dual<N>& b, double xmin, double xmax) {
  const double x = bisection(d.v, c.v, b.v, xmin, xmax);
  Dual<N> r(x);
  const double f0 = cubic(d.v, c.v, b.v, xmin), f1 = cubic(d.v, c.v, b.v, xmax);
  if (signbit(f0) == signbit(f1)) return r;  // an end point: locally constant
  const double fp = 3. * x * x + 2. * b.v * x + c.v;
  if (fp == 0.) return r;
  for (int k = 0; k < N; ++k) r.d[k] = -SWE_DIV(d.d[k] + c.d[k] * x + b.d[k] * x * x, fp);
  return r;
}
SWE_HD double bisection_t(double d, double c, double b, double xmin, double xmax) {
  return bisection(d, c, b, xmin, xmax);
}
// bisection_t when the forward pass already found the root x: the same value
// and implicit-function derivatives without repeating the bisection.
template <int N>
SWE_HD Dual<N> bisection_root_t(const Dual<N>& d, const Dual<N>& c, const Dual<N>& b, double xmin, double xmax,
                                double x) {
  Dual<N> r(x);
  const double f0 = cubic(d.v, c.v, b.v, xmin), f1 = cubic(d.v, c.v, b.v, xmax);
  if (signbit(f0) == signbit(f1)) return r;
  const double fp = 3. * x * x + 2. * b.v * x + c.v;
  if (fp == 0.) return r;
  for (int k = 0; k < N; ++k) r.d[k] = -SWE_DIV(d.d[k] + c.d[k] * x + b.d[k] * x * x, fp);
  return r;
}

// cube root with derivative (1/3) x^(-2/3); 0 at 0
SWE_HD double tcbrt(double x) { return cbrt_rn(x); }
template <int N>
SWE_HD Dual<N> tcbrt(const Dual<N>& a) {
  const double y = cbrt_rn(a.v);
  Dual<N> r(y);
  const double g = (y != 0.) ? SWE_DIV(1., 3. * y * y) : 0.;
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * g;
  return r;
}

}  // namespace swe
