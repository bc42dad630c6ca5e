// swe_physics.cuh -- point-wise physics of the SWE_FVM step, shared by the
// host-side geometry precompute and the sm_103a kernels.
//
// Every function restates one piece of the reference (NikitaMatckevich/
// SWE_FVM) with the same operation order, so that the device results match
// the CPU restatement bit for bit when the kernels are built without FMA
// contraction.  g = 1 throughout (the reference is nondimensional).
#pragma once

#include <cmath>
#include <cstdint>

#include "swe_fp64.cuh"

#if defined(__CUDACC__)
#define SWE_HD __host__ __device__ __forceinline__
#else
#define SWE_HD inline
#endif

namespace swe {

// Division and square root: the exact integer-pipe routines on the device
// (bit-identical to IEEE a / b and sqrt), the IEEE operators on the host.
#if defined(__CUDA_ARCH__)
#define SWE_DIV(a, b) ::swe::ddiv_rn((a), (b))
#define SWE_SQRT(x) ::swe::dsqrt_rn((x))
#else
#define SWE_DIV(a, b) ((a) / (b))
#define SWE_SQRT(x) std::sqrt((x))
#endif
// 0.5 x and -x (exact operations; on the device without FP64 instructions)
#if defined(__CUDA_ARCH__)
#define SWE_HALF(x) ::swe::dhalf_rn((x))
#define SWE_NEG(x) ::swe::dneg((x))
#else
#define SWE_HALF(x) (0.5 * (x))
#define SWE_NEG(x) (-(x))
#endif

// include/Includes.h:30
constexpr double kTol = 1e-13;
// include/Bathymetry.h:5-8
constexpr double kWetDepth = 1e-12;
// include/Fluxes.h:28,37,73
constexpr double kMinCapture = 1e-10;
// include/Assigners.h:30-32
constexpr double kEta1 = 1e-3;
constexpr double kEta2 = 1e-6;
constexpr double kEta4 = 1e-12;
constexpr double kSqrt2 = 1.4142135623730951;  // std::sqrt(2), correctly rounded

// ------------------------------------------------------------ comparisons
// On GB300 a warp-wide FP64 instruction, compares included, occupies the
// FP64 pipe for ~64 cycles, while the integer pipe issues one per cycle.  On the
// device every comparison therefore goes through integer keys: for non-NaN
// doubles, key(x) = (bits < 0) ? -(bits & 0x7FF..F) : bits is monotone and maps
// -0 and +0 to the same key, so a < b <=> key(a) < key(b) exactly.  (A NaN
// anywhere makes the state non-finite, which the update kernel reports.)  The
// host keeps the IEEE comparisons: the two agree on every non-NaN input.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ long long fkey(double x) {
  const long long i = dbits(x);
  return i < 0 ? -(i & 0x7FFFFFFFFFFFFFFFll) : i;
}
__device__ __forceinline__ long long fbits(double x) { return dbits(x); }
SWE_HD bool dlt(double a, double b) { return fkey(a) < fkey(b); }
SWE_HD bool dle(double a, double b) { return fkey(a) <= fkey(b); }
// x > c and x < c for a constant c > 0: the signed bit patterns order them
SWE_HD bool dgtc(double x, double c) { return fbits(x) > fbits(c); }
SWE_HD bool dltc(double x, double c) { return fbits(x) < fbits(c); }
// x > 0 and x >= 0
SWE_HD bool dgt0(double x) { return fbits(x) > 0; }
SWE_HD bool dge0(double x) { return fkey(x) >= 0; }
#else
SWE_HD bool dlt(double a, double b) { return a < b; }
SWE_HD bool dle(double a, double b) { return a <= b; }
SWE_HD bool dgtc(double x, double c) { return x > c; }
SWE_HD bool dltc(double x, double c) { return x < c; }
SWE_HD bool dgt0(double x) { return x > 0.; }
SWE_HD bool dge0(double x) { return x >= 0.; }
#endif

SWE_HD bool is_wet(double h) { return dgtc(h, kWetDepth); }
// std::min / std::max (first argument kept on ties)
SWE_HD double smin(double a, double b) { return dlt(b, a) ? b : a; }
SWE_HD double smax(double a, double b) { return dlt(a, b) ? b : a; }

// ---------------------------------------------------------------- geometry
// src/PointOperations.cpp:42-48: slope (gx, gy) of the plane through three
// points, 2x2 partial-pivot LU (pivot: first row with the largest |a_i0|).
SWE_HD void plane_gradient(double p0x, double p0y, double p0z, double p1x, double p1y, double p1z, double p2x,
                           double p2y, double p2z, double* gx, double* gy) {
  double a00 = p1x - p0x, a01 = p1y - p0y, b0 = p1z - p0z;
  double a10 = p2x - p0x, a11 = p2y - p0y, b1 = p2z - p0z;
  if (dlt(fabs(a00), fabs(a10))) {
    double t;
    t = a00; a00 = a10; a10 = t;
    t = a01; a01 = a11; a11 = t;
    t = b0; b0 = b1; b1 = t;
  }
  double l10 = a10;
  if (a00 != 0.) l10 = SWE_DIV(a10, a00);
  double u11 = a11 - l10 * a01;
  double y1 = b1 - l10 * b0;
  double x1 = SWE_DIV(y1, u11);
  double x0 = SWE_DIV(b0 - a01 * x1, a00);
  *gx = x0;
  *gy = x1;
}

// (int)log2(x) for finite x > 0, truncated toward zero, from the exponent bits
// (src/PointOperations.cpp:33).
SWE_HD int trunc_log2(double x) {
  int e;
  double m = frexp(x, &e);
  if (m == 0.5) return e - 1;
  return (e >= 1) ? e - 1 : e;
}

// Correctly rounded cube root (round to nearest, ties to even) for the
// PartWet1 level (src/MUSCLObject.cpp:103).  The math libraries' cbrt are
// faithful, not correctly rounded, and the CUDA and host ones differ in the
// last bit; this one is exact on both.  Method: x = Mx 2^E with a 53-bit
// integer Mx; N = Mx 2^t with t in {107, 108, 109} chosen so that 3 | (E - t)
// and N in [2^159, 2^162); Y = floor(cbrt(N)) in [2^53, 2^54) is found from a
// library estimate corrected with exact 192-bit integer cubes; its lowest bit
// and the remainder N - Y^3 round it to 53 bits.
struct U192 {
  unsigned long long w[3];  // little-endian limbs
};
SWE_HD U192 u192_cube(unsigned long long y) {
  // y < 2^55: y^2 < 2^110 fits 128 bits, y^3 < 2^165 fits 192 bits
  unsigned __int128 y2 = (unsigned __int128)y * y;
  unsigned __int128 lo = (unsigned __int128)(unsigned long long)y2 * y;
  unsigned __int128 hi = (unsigned __int128)(unsigned long long)(y2 >> 64) * y;
  U192 r;
  r.w[0] = (unsigned long long)lo;
  unsigned __int128 mid = (lo >> 64) + (unsigned long long)hi;
  r.w[1] = (unsigned long long)mid;
  r.w[2] = (unsigned long long)((mid >> 64) + (hi >> 64));
  return r;
}
SWE_HD int u192_cmp(const U192& a, const U192& b) {
  for (int k = 2; k >= 0; --k) {
    if (a.w[k] < b.w[k]) return -1;
    if (a.w[k] > b.w[k]) return 1;
  }
  return 0;
}
SWE_HD double cbrt_rn(double x) {
  if (!(x == x) || x == 0. || isinf(x)) return x + x;  // NaN, +-0, +-inf
  const bool neg = x < 0.;
  double ax = neg ? -x : x;
  int scale = 0;
  if (ax < 2.2250738585072014e-308) {  // subnormal: scale by 2^54
    ax = ax * 18014398509481984.0;
    scale = -18;
  }
  int e;
  const double m = frexp(ax, &e);                                  // ax = m 2^e, m in [0.5, 1)
  const unsigned long long Mx = (unsigned long long)ldexp(m, 53);  // exact 53-bit integer
  const int E = e - 53;                                            // ax = Mx 2^E
  int t = 107;
  while (((E - t) % 3 + 3) % 3 != 0) ++t;
  // N = Mx 2^t as 192 bits
  U192 N;
  {
    const int word = t / 64, bit = t % 64;
    N.w[0] = N.w[1] = N.w[2] = 0ull;
    N.w[word] = Mx << bit;
    if (bit && word + 1 < 3) N.w[word + 1] = Mx >> (64 - bit);
  }
  // estimate: cbrt(Mx 2^t) = cbrt(Mx) 2^(t/3)
  const double est = ldexp(cbrt((double)Mx * ldexp(1.0, t % 3)), t / 3);
  unsigned long long Y = (unsigned long long)est;
  if (Y < (1ull << 53)) Y = 1ull << 53;
  if (Y >= (1ull << 54)) Y = (1ull << 54) - 1;
  for (int it = 0; it < 64 && u192_cmp(u192_cube(Y), N) > 0; ++it) --Y;
  for (int it = 0; it < 64 && u192_cmp(u192_cube(Y + 1), N) <= 0; ++it) ++Y;
  const bool sticky = u192_cmp(u192_cube(Y), N) != 0;
  unsigned long long R = Y >> 1;
  if ((Y & 1ull) && (sticky || (R & 1ull))) ++R;
  const double r = ldexp((double)R, (E - t) / 3 + 1 + scale);
  return neg ? -r : r;
}

// include/CubicPolyMath.h:13-15: x^3 + b x^2 + c x + d
SWE_HD double cubic(double d, double c, double b, double x) { return x * x * x + b * x * x + c * x + d; }

// src/PointOperations.cpp:26-40.  f(xmin) is carried between iterations
// instead of re-evaluated: the same function of the same argument.
SWE_HD double bisection(double d, double c, double b, double xmin, double xmax) {
  double fmin_ = cubic(d, c, b, xmin);
  double fmax_ = cubic(d, c, b, xmax);
  if (signbit(fmin_) == signbit(fmax_)) return dlt(fabs(fmin_), fabs(fmax_)) ? xmin : xmax;
  int n = 50 + trunc_log2(xmax - xmin);
  double x = 0.;
  bool smin_ = signbit(fmin_);
  for (int it = 0; it <= n; it++) {
    x = SWE_HALF(xmin + xmax);
    double fx = cubic(d, c, b, x);
    bool sx = signbit(fx);
    if (smin_ != sx) {
      xmax = x;
    } else {
      xmin = x;
      smin_ = sx;
    }
  }
  return x;
}

// --------------------------------------------------------------- assigners
// src/Assigners.cpp:8-20: PrimAssigner (edge writes)
SWE_HD void prim_assign(double b, double w, double u, double v, double* ow, double* ou, double* ov) {
  double h = w - b;
  if (!is_wet(h)) {
    *ow = b; *ou = 0.; *ov = 0.;
    return;
  }
  if (dltc(h, kEta1)) {
    double s = SWE_DIV(kSqrt2 * h, SWE_SQRT(h * h + kEta2));
    u *= s;
    v *= s;
  }
  *ow = w; *ou = u; *ov = v;
}

// src/Assigners.cpp:28-44: ConsAssigner (cell writes)
SWE_HD void cons_assign(double b, double h, double hu, double hv, double* ow, double* ou, double* ov) {
  if (!is_wet(h)) {
    *ow = b; *ou = 0.; *ov = 0.;
    return;
  }
  double ih;
  if (dltc(h, kEta1)) ih = SWE_DIV(kSqrt2 * h, SWE_SQRT(h * h * h * h + kEta4));
  else ih = SWE_DIV(1., h);
  *ow = h + b;
  *ou = hu * ih;
  *ov = hv * ih;
}

// -------------------------------------------------------------- edge flux
// include/SpaceDisc.h:4-18: F.n of U = (h, hu, hv), g = 1
SWE_HD void elem_flux(double nx, double ny, double h, double hu, double hv, double* f) {
  f[0] = 0.; f[1] = 0.; f[2] = 0.;
  if (is_wet(h)) {
    double hveln = hu * nx + hv * ny;
    f[0] = hveln;
    const double q = SWE_DIV(hveln, h);
    const double p = SWE_HALF(h) * h;  // 0.5 h h
    f[1] = q * hu + p * nx;
    f[2] = q * hv + p * ny;
  }
}

// Wave-speed plugins (src/Fluxes.cpp:5-26).  speeds() returns the pair the
// reference's Array<2> holds.
// What a flux evaluation can leave for its reverse: the wave speeds'
// intermediates and u* (the discrete adjoint's recompute stores them, see
// swe_flux_adjoint.cuh).  NoTape records nothing and compiles away.
struct NoTape {
  SWE_HD void speeds(double, double, double, double, double, double) const {}
  SWE_HD void ustar(double) const {}
};
// Edge e's intermediates into t[k * E + e]: cl, cr, uRoe, cRoe, a0, a1, u*.
struct EdgeTape {
  double* t;
  int E, e;
  SWE_HD void speeds(double cl, double cr, double uRoe, double cRoe, double a0, double a1) const {
    t[e] = cl;
    t[E + e] = cr;
    t[2 * E + e] = uRoe;
    t[3 * E + e] = cRoe;
    t[4 * E + e] = a0;
    t[5 * E + e] = a1;
  }
  SWE_HD void ustar(double us) const { t[6 * E + e] = us; }
};

struct Rusanov {
  static constexpr int id = 0;
  template <class T>
  SWE_HD static void speeds(double ul, double hl, double ur, double hr, double* a0, double* a1, const T& tape) {
    double cl = SWE_SQRT(hl), cr = SWE_SQRT(hr);
    double ap = smax(fabs(ul) + cl, fabs(ur) + cr);
    *a0 = -ap;
    *a1 = ap;
    tape.speeds(cl, cr, 0., 0., *a0, *a1);
  }
  SWE_HD static void speeds(double ul, double hl, double ur, double hr, double* a0, double* a1) {
    speeds(ul, hl, ur, hr, a0, a1, NoTape{});
  }
};
struct Davis {
  static constexpr int id = 1;
  template <class T>
  SWE_HD static void speeds(double ul, double hl, double ur, double hr, double* a0, double* a1, const T& tape) {
    double cl = SWE_SQRT(hl), cr = SWE_SQRT(hr);
    *a0 = smin(ul - cl, ur - cr);
    *a1 = smax(ul + cl, ur + cr);
    tape.speeds(cl, cr, 0., 0., *a0, *a1);
  }
  SWE_HD static void speeds(double ul, double hl, double ur, double hr, double* a0, double* a1) {
    speeds(ul, hl, ur, hr, a0, a1, NoTape{});
  }
};
struct Einfeldt {
  static constexpr int id = 2;
  template <class T>
  SWE_HD static void speeds(double ul, double hl, double ur, double hr, double* a0, double* a1, const T& tape) {
    double cl = SWE_SQRT(hl), cr = SWE_SQRT(hr);
    double uRoe = SWE_DIV(cl * ul + cl * ur, cl + cr);  // the reference's cl * ur
    double cRoe = SWE_SQRT(SWE_HALF(hl + hr));
    *a0 = smin(ul - cl, uRoe - cRoe);
    *a1 = smax(ur + cr, uRoe + cRoe);
    tape.speeds(cl, cr, uRoe, cRoe, *a0, *a1);
  }
  SWE_HD static void speeds(double ul, double hl, double ur, double hr, double* a0, double* a1) {
    speeds(ul, hl, ur, hr, a0, a1, NoTape{});
  }
};

// Everything a flux plugin reads about one interior edge: the geometry of the
// edge seen from its owner ("from", include/Fluxes.h:20,62-63) and the two
// reconstructed interface states.
struct EdgeGeom {
  double nx, ny;  // Domain::Norm(e, from)
  double tx, ty;  // Domain::Tang(e, from)
  double b;       // edge-centre bathymetry
  double lmin;    // min(2 A_from / L, 2 A_to / L)
};
struct SideState {
  double w, u, v;  // interface primitive values (EdgeField slot)
};

// Fluxes::HLL<W> (include/Fluxes.h:14-54).  *lw receives the edge's
// length-to-wavespeed ratio, or is left alone when the edge does not update it.
template <class W>
struct HLL {
  static constexpr int id = 0;
  SWE_HD static void eval(const EdgeGeom& g, const SideState& L, const SideState& R, double cor, double* lw,
                          double* F) {
    eval(g, L, R, cor, lw, F, NoTape{});
  }
  template <class T>
  SWE_HD static void eval(const EdgeGeom& g, const SideState& L, const SideState& R, double cor, double* lw,
                          double* F, const T& tape) {
    double ul = L.u * g.nx + L.v * g.ny;
    double hl = L.w - g.b;
    double ur = R.u * g.nx + R.v * g.ny;
    double hr = R.w - g.b;
    F[0] = 0.; F[1] = 0.; F[2] = 0.;
    if (!dgtc(hl + hr, kMinCapture)) return;
    double a0, a1;
    W::speeds(ul, hl, ur, hr, &a0, &a1, tape);
    double al = smin(0., a0);
    double ar = smax(0., a1);
    if (!dgtc(ar - al, kMinCapture)) return;
    *lw = SWE_DIV(g.lmin, fabs(cor) + smax(-al, ar));
    double Ul[3] = {hl, hl * L.u, hl * L.v};
    double Ur[3] = {hr, hr * R.u, hr * R.v};
    double Fl[3], Fr[3];
    elem_flux(g.nx, g.ny, Ul[0], Ul[1], Ul[2], Fl);
    elem_flux(g.nx, g.ny, Ur[0], Ur[1], Ur[2], Fr);
#pragma unroll
    for (int q = 0; q < 3; ++q) F[q] = SWE_DIV(ar * Fl[q] - al * Fr[q] + (al * ar) * (Ur[q] - Ul[q]), ar - al);
  }
};

// Fluxes::HLLC<W> (include/Fluxes.h:56-111)
template <class W>
struct HLLC {
  static constexpr int id = 1;
  SWE_HD static void eval(const EdgeGeom& g, const SideState& L, const SideState& R, double cor, double* lw,
                          double* F) {
    eval(g, L, R, cor, lw, F, NoTape{});
  }
  template <class T>
  SWE_HD static void eval(const EdgeGeom& g, const SideState& L, const SideState& R, double cor, double* lw,
                          double* F, const T& tape) {
    double ul = L.u * g.nx + L.v * g.ny;
    double hl = L.w - g.b;
    double ur = R.u * g.nx + R.v * g.ny;
    double hr = R.w - g.b;
    F[0] = 0.; F[1] = 0.; F[2] = 0.;
    if (!dgtc(hl + hr, kMinCapture)) return;
    double al, ar;
    W::speeds(ul, hl, ur, hr, &al, &ar, tape);
    // (ar - ur) hr = hr (ar - ur) and (al - ul) hl = hl (al - ul) bit for bit:
    // each product is formed once for u* and the star depth
    const double hrA = (ar - ur) * hr, hlB = (al - ul) * hl;
    double ustar = hrA * ur - hlB * ul + SWE_HALF(hl * hl - hr * hr);
    ustar = SWE_DIV(ustar, hrA - hlB);
    tape.ustar(ustar);
    *lw = SWE_DIV(g.lmin, fabs(cor) + smax(kTol, smax(al, ar)));
    // u* <= 0: the right star state, else the left one.  The side is picked
    // first and the shared formula evaluated once, so a warp whose edges take
    // both sides issues it once (the operations per side are the reference's).
    const bool right = !dgt0(ustar);
    const double hx = right ? hr : hl, ux = right ? R.u : L.u, vx = right ? R.v : L.v;
    const double ax = right ? ar : al, hxa = right ? hrA : hlB;  // hx (ax - u_n,x)
    const double vt = ux * g.tx + vx * g.ty;  // tangential velocity of that side
    double Ux[3] = {hx, hx * ux, hx * vx};
    double us = vt * g.tx + ustar * g.ty;
    double vs = vt * g.nx + ustar * g.ny;
    double hs = SWE_DIV(hxa, ax - ustar);
    double Us[3] = {hs, hs * us, hs * vs};
    double Fx[3];
    elem_flux(g.nx, g.ny, Ux[0], Ux[1], Ux[2], Fx);
    double s = right ? smax(0., ar) : smin(0., al);
#pragma unroll
    for (int q = 0; q < 3; ++q) F[q] = Fx[q] + s * (Us[q] - Ux[q]);
  }
};

// ------------------------------------------------------- ordered doubles
// Monotone map of doubles to unsigned 64-bit keys (for non-NaN values), so
// that integer atomicMax / atomicMin give the exact floating-point max / min.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned long long order_key(double d) {
  const unsigned long long u = (unsigned long long)dbits(d);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double order_val(unsigned long long k) {
  return dfrom((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}
#else
SWE_HD unsigned long long order_key(double d) {
  union {
    double d;
    unsigned long long u;
  } c;
  c.d = d;
  return (c.u >> 63) ? ~c.u : (c.u | 0x8000000000000000ull);
}
SWE_HD double order_val(unsigned long long k) {
  union {
    double d;
    unsigned long long u;
  } c;
  c.u = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return c.d;
}
#endif

}  // namespace swe
