// swe_flux_adjoint.cuh -- hand-written reverse of the flux plugins
// (include/Fluxes.h:14-111, src/Fluxes.cpp:5-26, include/SpaceDisc.h:4-18).
//
// flux_reverse() recomputes the forward flux of one interior edge, keeping its
// intermediates, and propagates the adjoint lF of (F0, F1, F2) back to the two
// interface states and the edge bathymetry, following the branches the forward
// took.  It matches the forward-mode Jacobian of flux_t (swe_dual.cuh); the
// self-test swe_selftest_flux_adjoint compares the two.
//
// Every value that steers a branch (depths, normal velocities, wave speeds,
// u*) is recomputed with the forward's own operations, so it is bit-identical
// to the forward pass.  Quantities that only feed derivatives use explicit
// fused multiply-adds: the library is compiled without FMA contraction (the
// forward must round like the reference), and one DFMA costs the FP64 pipe as
// much as one DMUL.
#pragma once

#include "swe_physics.cuh"

namespace swe {

// Forward wave speeds (src/Fluxes.cpp:5-26) with the intermediates the reverse
// reads; the same operations as the plugins' speeds().
struct WsFwd {
  double cl, cr, S, uRoe, cRoe, a0, a1;
};
SWE_HD WsFwd ws_forward(int ws, double ul, double hl, double ur, double hr) {
  WsFwd f;
  f.cl = SWE_SQRT(hl);
  f.cr = SWE_SQRT(hr);
  f.S = 0.;
  f.uRoe = 0.;
  f.cRoe = 0.;
  if (ws == 0) {
    const double ap = smax(fabs(ul) + f.cl, fabs(ur) + f.cr);
    f.a0 = -ap;
    f.a1 = ap;
  } else if (ws == 1) {
    f.a0 = smin(ul - f.cl, ur - f.cr);
    f.a1 = smax(ul + f.cl, ur + f.cr);
  } else {
    f.S = f.cl + f.cr;
    f.uRoe = SWE_DIV(f.cl * ul + f.cl * ur, f.S);
    f.cRoe = SWE_SQRT(0.5 * (hl + hr));
    f.a0 = smin(ul - f.cl, f.uRoe - f.cRoe);
    f.a1 = smax(ur + f.cr, f.uRoe + f.cRoe);
  }
  return f;
}

// ElemFlux(n, (h, hu, hv)) (include/SpaceDisc.h:4-18) for derivative use only
SWE_HD void elem_flux_fma(double nx, double ny, double h, double hu, double hv, double ih, double* f) {
  f[0] = 0.;
  f[1] = 0.;
  f[2] = 0.;
  if (is_wet(h)) {
    const double hveln = fma(hu, nx, hv * ny);
    const double q = hveln * ih;
    const double p = 0.5 * h * h;
    f[0] = hveln;
    f[1] = fma(q, hu, p * nx);
    f[2] = fma(q, hv, p * ny);
  }
}

// ElemFlux reverse: adds to lh, lhu, lhv (ih = 1 / h)
SWE_HD void elem_flux_rev(double nx, double ny, double h, double hu, double hv, double ih, const double* lf,
                          double* lh, double* lhu, double* lhv) {
  if (!is_wet(h)) return;
  const double q = fma(hu, nx, hv * ny) * ih;
  const double lqh = fma(lf[1], hu, lf[2] * hv) * ih;
  const double lhveln = lf[0] + lqh;
  *lhu = fma(lf[1], q, fma(lhveln, nx, *lhu));
  *lhv = fma(lf[2], q, fma(lhveln, ny, *lhv));
  *lh = fma(-lqh, q, fma(fma(lf[1], nx, lf[2] * ny), h, *lh));
}

// wave-speed reverse: given la0, la1, adds to lul, lhl, lur, lhr
SWE_HD void wavespeeds_rev(int ws, const WsFwd& f, double ul, double ur, double la0, double la1, double* lul,
                           double* lhl, double* lur, double* lhr) {
  double lcl = 0., lcr = 0.;
  if (ws == 0) {
    const double lap = la1 - la0;
    if (dlt(fabs(ul) + f.cl, fabs(ur) + f.cr)) {  // smax picked the right side
      *lur += signbit(ur) ? -lap : lap;
      lcr += lap;
    } else {
      *lul += signbit(ul) ? -lap : lap;
      lcl += lap;
    }
  } else if (ws == 1) {
    if (dlt(ur - f.cr, ul - f.cl)) {
      *lur += la0;
      lcr -= la0;
    } else {
      *lul += la0;
      lcl -= la0;
    }
    if (dlt(ul + f.cl, ur + f.cr)) {
      *lur += la1;
      lcr += la1;
    } else {
      *lul += la1;
      lcl += la1;
    }
  } else {
    double luRoe = 0., lcRoe = 0.;
    if (dlt(f.uRoe - f.cRoe, ul - f.cl)) {
      luRoe += la0;
      lcRoe -= la0;
    } else {
      *lul += la0;
      lcl -= la0;
    }
    if (dlt(ur + f.cr, f.uRoe + f.cRoe)) {
      luRoe += la1;
      lcRoe += la1;
    } else {
      *lur += la1;
      lcr += la1;
    }
    if (f.cRoe > 0.) {  // cRoe = sqrt((hl + hr) / 2)
      const double lm = lcRoe * SWE_DIV(0.25, f.cRoe);
      *lhl += lm;
      *lhr += lm;
    }
    // uRoe = cl (ul + ur) / S, S = cl + cr
    const double lN = luRoe * SWE_DIV(1., f.S);
    const double lS = -lN * f.uRoe;
    lcl = fma(lN, ul + ur, lcl + lS);
    *lul = fma(lN, f.cl, *lul);
    *lur = fma(lN, f.cl, *lur);
    lcr += lS;
  }
  if (f.cl > 0.) *lhl = fma(lcl, SWE_DIV(0.5, f.cl), *lhl);
  if (f.cr > 0.) *lhr = fma(lcr, SWE_DIV(0.5, f.cr), *lhr);
}

// Reverse of one interior edge's flux.  g: edge geometry; L, R: interface
// primitives; lF: adjoint of (F0, F1, F2).  Adds to lL[3], lR[3] (w, u, v)
// and *lb (edge bathymetry).  tape: null, or the forward's stored wave-speed
// intermediates and u* of this edge (EdgeTape layout, tape[k E + e]), which
// then are not recomputed.
SWE_HD void flux_reverse(int flux, int ws, const EdgeGeom& g, const SideState& L, const SideState& R,
                         const double* lF, double* lL, double* lR, double* lb, const double* tape = nullptr,
                         int E = 0, int e = 0) {
  const double nx = g.nx, ny = g.ny, tx = g.tx, ty = g.ty;
  const double ul = L.u * nx + L.v * ny;
  const double hl = L.w - g.b;
  const double ur = R.u * nx + R.v * ny;
  const double hr = R.w - g.b;
  if (!dgtc(hl + hr, kMinCapture)) return;
  double lul = 0., lhl = 0., lur = 0., lhr = 0., lvl = 0., lvr = 0.;
  double lLu = 0., lLv = 0., lRu = 0., lRv = 0.;
  WsFwd f;
  if (tape) {
    f.cl = tape[e];
    f.cr = tape[E + e];
    f.S = f.cl + f.cr;
    f.uRoe = tape[2 * E + e];
    f.cRoe = tape[3 * E + e];
    f.a0 = tape[4 * E + e];
    f.a1 = tape[5 * E + e];
  } else {
    f = ws_forward(ws, ul, hl, ur, hr);
  }
  if (flux == 0) {
    const double a0 = f.a0, a1 = f.a1;
    const double al = smin(0., a0);
    const double ar = smax(0., a1);
    if (!dgtc(ar - al, kMinCapture)) return;
    const double ihl = is_wet(hl) ? SWE_DIV(1., hl) : 0.;
    const double ihr = is_wet(hr) ? SWE_DIV(1., hr) : 0.;
    const double Ul[3] = {hl, hl * L.u, hl * L.v};
    const double Ur[3] = {hr, hr * R.u, hr * R.v};
    double Fl[3], Fr[3];
    elem_flux_fma(nx, ny, Ul[0], Ul[1], Ul[2], ihl, Fl);
    elem_flux_fma(nx, ny, Ur[0], Ur[1], Ur[2], ihr, Fr);
    const double iDn = SWE_DIV(1., ar - al);
    const double alar = al * ar;
    double lG[3], dU[3];
    double lDn = 0.;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      dU[q] = Ur[q] - Ul[q];
      const double F = fma(ar, Fl[q], fma(-al, Fr[q], alar * dU[q])) * iDn;
      lG[q] = lF[q] * iDn;
      lDn = fma(-lG[q], F, lDn);
    }
    double lar = lDn, lal = -lDn;
    double lFl[3], lFr[3], lUl[3], lUr[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      lar = fma(lG[q], fma(al, dU[q], Fl[q]), lar);
      lal = fma(lG[q], fma(ar, dU[q], -Fr[q]), lal);
      lFl[q] = ar * lG[q];
      lFr[q] = -al * lG[q];
      lUr[q] = alar * lG[q];
      lUl[q] = -lUr[q];
    }
    elem_flux_rev(nx, ny, Ul[0], Ul[1], Ul[2], ihl, lFl, &lUl[0], &lUl[1], &lUl[2]);
    elem_flux_rev(nx, ny, Ur[0], Ur[1], Ur[2], ihr, lFr, &lUr[0], &lUr[1], &lUr[2]);
    const double la0 = dlt(a0, 0.) ? lal : 0.;
    const double la1 = dlt(0., a1) ? lar : 0.;
    wavespeeds_rev(ws, f, ul, ur, la0, la1, &lul, &lhl, &lur, &lhr);
    lhl = fma(lUl[1], L.u, fma(lUl[2], L.v, lhl + lUl[0]));
    lLu = fma(lUl[1], hl, lLu);
    lLv = fma(lUl[2], hl, lLv);
    lhr = fma(lUr[1], R.u, fma(lUr[2], R.v, lhr + lUr[0]));
    lRu = fma(lUr[1], hr, lRu);
    lRv = fma(lUr[2], hr, lRv);
  } else {
    const double al = f.a0, ar = f.a1;
    const double A = ar - ur, B = al - ul;
    // u* with the forward's operations (its sign picks the star side), or the
    // forward's own value
    const double D = hr * A - hl * B;
    const double us = tape ? tape[6 * E + e] : SWE_DIV(A * hr * ur - B * hl * ul + 0.5 * (hl * hl - hr * hr), D);
    double lus = 0., lA = 0., lB = 0., lar = 0., lal = 0.;
    // the star side the forward took (u* <= 0: right), evaluated once and
    // scattered by selects, so a warp whose edges take both sides issues it once
    const bool right = !dgt0(us);
    const SideState& X = right ? R : L;
    const double hx = right ? hr : hl, Kx = right ? A : B, ax = right ? ar : al;
    const double vtx = fma(X.u, tx, X.v * ty);
    const double ihx = is_wet(hx) ? SWE_DIV(1., hx) : 0.;
    const double Ux[3] = {hx, hx * X.u, hx * X.v};
    const double uxs = fma(vtx, tx, us * ty);
    const double vys = fma(vtx, nx, us * ny);
    const double iY = SWE_DIV(1., ax - us);
    const double hs = hx * Kx * iY;
    const double Us[3] = {hs, hs * uxs, hs * vys};
    const double sx = right ? smax(0., ar) : smin(0., al);
    double lsx = 0., lUx[3], lUs[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      lsx = fma(lF[q], Us[q] - Ux[q], lsx);
      lUs[q] = sx * lF[q];
      lUx[q] = -lUs[q];
    }
    double lax = (right ? dlt(0., ar) : dlt(al, 0.)) ? lsx : 0.;
    elem_flux_rev(nx, ny, Ux[0], Ux[1], Ux[2], ihx, lF, &lUx[0], &lUx[1], &lUx[2]);
    const double lhs = fma(lUs[1], uxs, fma(lUs[2], vys, lUs[0]));
    const double luxs = lUs[1] * hs, lvys = lUs[2] * hs;
    const double lX = lhs * iY, lY = -lX * hs;
    double lhx = lX * Kx;
    const double lKx = lX * hx;
    lax += lY;
    lus -= lY;
    const double lvtx = fma(luxs, tx, lvys * nx);
    lus = fma(luxs, ty, fma(lvys, ny, lus));
    lhx = fma(lUx[1], X.u, fma(lUx[2], X.v, lhx + lUx[0]));
    const double lux = lUx[1] * hx, lvx = lUx[2] * hx;
    if (right) {
      lhr += lhx;
      lA += lKx;
      lar += lax;
      lvr = lvtx;
      lRu += lux;
      lRv += lvx;
    } else {
      lhl += lhx;
      lB += lKx;
      lal += lax;
      lvl = lvtx;
      lLu += lux;
      lLv += lvx;
    }
    // us = N / D
    const double lN = lus * SWE_DIV(1., D);
    const double lD = -lN * us;
    lhr = fma(lD, A, lhr);
    lA = fma(lD, hr, lA);
    lhl = fma(-lD, B, lhl);
    lB = fma(-lD, hl, lB);
    const double lNhr = lN * hr, lNhl = lN * hl;
    lA = fma(lNhr, ur, lA);
    lhr = fma(lN * A, ur, lhr);
    lur = fma(lNhr, A, lur);
    lB = fma(-lNhl, ul, lB);
    lhl = fma(-lN * B, ul, lhl);
    lul = fma(-lNhl, B, lul);
    lhl += lNhl;
    lhr -= lNhr;
    lar += lA;
    lur -= lA;
    lal += lB;
    lul -= lB;
    wavespeeds_rev(ws, f, ul, ur, lal, lar, &lul, &lhl, &lur, &lhr);
  }
  lLu = fma(lul, nx, fma(lvl, tx, lLu));
  lLv = fma(lul, ny, fma(lvl, ty, lLv));
  lRu = fma(lur, nx, fma(lvr, tx, lRu));
  lRv = fma(lur, ny, fma(lvr, ty, lRv));
  lL[0] += lhl;
  lL[1] += lLu;
  lL[2] += lLv;
  lR[0] += lhr;
  lR[1] += lRu;
  lR[2] += lRv;
  *lb -= lhl + lhr;
}

}  // namespace swe
