// swe_flux_adjoint.cuh -- hand-written reverse of the flux plugins
// (include/Fluxes.h:14-111, src/Fluxes.cpp:5-26, include/SpaceDisc.h:4-18).
//
// flux_reverse() recomputes the forward flux of one interior edge, keeping its
// intermediates, and propagates the adjoint lF of (F0, F1, F2) back to the two
// interface states and the edge bathymetry, following the branches the forward
// took.  It matches the forward-mode Jacobian of flux_t (swe_dual.cuh); the
// self-test swe_selftest_flux_adjoint compares the two.
#pragma once

#include "swe_physics.cuh"

namespace swe {

// ElemFlux(n, (h, hu, hv)) reverse: adds to lh, lhu, lhv
SWE_HD void elem_flux_rev(double nx, double ny, double h, double hu, double hv, const double* lf, double* lh,
                          double* lhu, double* lhv) {
  if (!is_wet(h)) return;
  const double hveln = hu * nx + hv * ny;
  const double q = SWE_DIV(hveln, h);
  const double lq = lf[1] * hu + lf[2] * hv;
  const double lhveln = lf[0] + SWE_DIV(lq, h);
  *lhu += lf[1] * q + lhveln * nx;
  *lhv += lf[2] * q + lhveln * ny;
  *lh += -SWE_DIV(lq * q, h) + (lf[1] * nx + lf[2] * ny) * h;
}

// wave-speed reverse: given la0, la1, adds to lul, lhl, lur, lhr
SWE_HD void wavespeeds_rev(int ws, double ul, double hl, double ur, double hr, double la0, double la1, double* lul,
                           double* lhl, double* lur, double* lhr) {
  const double cl = SWE_SQRT(hl), cr = SWE_SQRT(hr);
  double lcl = 0., lcr = 0.;
  if (ws == 0) {
    const double xl = fabs(ul) + cl, xr = fabs(ur) + cr;
    const double lap = la1 - la0;
    if (dlt(xl, xr)) {  // smax picked the right side
      *lur += signbit(ur) ? -lap : lap;
      lcr += lap;
    } else {
      *lul += signbit(ul) ? -lap : lap;
      lcl += lap;
    }
  } else if (ws == 1) {
    if (dlt(ur - cr, ul - cl)) {
      *lur += la0;
      lcr -= la0;
    } else {
      *lul += la0;
      lcl -= la0;
    }
    if (dlt(ul + cl, ur + cr)) {
      *lur += la1;
      lcr += la1;
    } else {
      *lul += la1;
      lcl += la1;
    }
  } else {
    const double S = cl + cr;
    const double uRoe = SWE_DIV(cl * ul + cl * ur, S);
    const double cRoe = SWE_SQRT(0.5 * (hl + hr));
    double luRoe = 0., lcRoe = 0.;
    if (dlt(uRoe - cRoe, ul - cl)) {
      luRoe += la0;
      lcRoe -= la0;
    } else {
      *lul += la0;
      lcl -= la0;
    }
    if (dlt(ur + cr, uRoe + cRoe)) {
      luRoe += la1;
      lcRoe += la1;
    } else {
      *lur += la1;
      lcr += la1;
    }
    if (cRoe > 0.) {
      const double lm = SWE_DIV(0.5 * lcRoe, cRoe);
      *lhl += 0.5 * lm;
      *lhr += 0.5 * lm;
    }
    const double lN = SWE_DIV(luRoe, S);
    const double lS = -SWE_DIV(luRoe * uRoe, S);
    lcl += lN * (ul + ur) + lS;
    *lul += lN * cl;
    *lur += lN * cl;
    lcr += lS;
  }
  if (cl > 0.) *lhl += SWE_DIV(0.5 * lcl, cl);
  if (cr > 0.) *lhr += SWE_DIV(0.5 * lcr, cr);
}

// Reverse of one interior edge's flux.  g: edge geometry; L, R: interface
// primitives; lF: adjoint of (F0, F1, F2).  Adds to lL[3], lR[3] (w, u, v)
// and *lb (edge bathymetry).
SWE_HD void flux_reverse(int flux, int ws, const EdgeGeom& g, const SideState& L, const SideState& R,
                         const double* lF, double* lL, double* lR, double* lb) {
  const double nx = g.nx, ny = g.ny, tx = g.tx, ty = g.ty;
  const double ul = L.u * nx + L.v * ny;
  const double hl = L.w - g.b;
  const double ur = R.u * nx + R.v * ny;
  const double hr = R.w - g.b;
  if (!dgtc(hl + hr, kMinCapture)) return;
  double lul = 0., lhl = 0., lur = 0., lhr = 0., lvl = 0., lvr = 0.;
  double lLu = 0., lLv = 0., lRu = 0., lRv = 0.;
  if (flux == 0) {
    double a0, a1;
    switch (ws) {
      case 0: Rusanov::speeds(ul, hl, ur, hr, &a0, &a1); break;
      case 1: Davis::speeds(ul, hl, ur, hr, &a0, &a1); break;
      default: Einfeldt::speeds(ul, hl, ur, hr, &a0, &a1); break;
    }
    const double al = smin(0., a0);
    const double ar = smax(0., a1);
    if (!dgtc(ar - al, kMinCapture)) return;
    const double Ul[3] = {hl, hl * L.u, hl * L.v};
    const double Ur[3] = {hr, hr * R.u, hr * R.v};
    double Fl[3], Fr[3];
    elem_flux(nx, ny, Ul[0], Ul[1], Ul[2], Fl);
    elem_flux(nx, ny, Ur[0], Ur[1], Ur[2], Fr);
    const double Dn = ar - al;
    double F[3], lG[3];
    double lDn = 0.;
    for (int q = 0; q < 3; ++q) {
      F[q] = SWE_DIV(ar * Fl[q] - al * Fr[q] + (al * ar) * (Ur[q] - Ul[q]), Dn);
      lG[q] = SWE_DIV(lF[q], Dn);
      lDn -= SWE_DIV(lF[q] * F[q], Dn);
    }
    double lar = lDn, lal = -lDn;
    double lFl[3], lFr[3], lUl[3], lUr[3];
    for (int q = 0; q < 3; ++q) {
      lar += lG[q] * (Fl[q] + al * (Ur[q] - Ul[q]));
      lal += lG[q] * (-Fr[q] + ar * (Ur[q] - Ul[q]));
      lFl[q] = ar * lG[q];
      lFr[q] = -al * lG[q];
      lUr[q] = (al * ar) * lG[q];
      lUl[q] = -(al * ar) * lG[q];
    }
    elem_flux_rev(nx, ny, Ul[0], Ul[1], Ul[2], lFl, &lUl[0], &lUl[1], &lUl[2]);
    elem_flux_rev(nx, ny, Ur[0], Ur[1], Ur[2], lFr, &lUr[0], &lUr[1], &lUr[2]);
    const double la0 = dlt(a0, 0.) ? lal : 0.;
    const double la1 = dlt(0., a1) ? lar : 0.;
    wavespeeds_rev(ws, ul, hl, ur, hr, la0, la1, &lul, &lhl, &lur, &lhr);
    lhl += lUl[0] + lUl[1] * L.u + lUl[2] * L.v;
    lLu += lUl[1] * hl;
    lLv += lUl[2] * hl;
    lhr += lUr[0] + lUr[1] * R.u + lUr[2] * R.v;
    lRu += lUr[1] * hr;
    lRv += lUr[2] * hr;
  } else {
    const double vl = L.u * tx + L.v * ty;
    const double vr = R.u * tx + R.v * ty;
    double al, ar;
    switch (ws) {
      case 0: Rusanov::speeds(ul, hl, ur, hr, &al, &ar); break;
      case 1: Davis::speeds(ul, hl, ur, hr, &al, &ar); break;
      default: Einfeldt::speeds(ul, hl, ur, hr, &al, &ar); break;
    }
    const double A = ar - ur, B = al - ul;
    double us = A * hr * ur - B * hl * ul + 0.5 * (hl * hl - hr * hr);
    const double N = us;
    const double D = hr * A - hl * B;
    us = SWE_DIV(us, D);
    (void)N;
    double lus = 0., lA = 0., lB = 0., lar = 0., lal = 0.;
    if (!dgt0(us)) {
      const double Ur[3] = {hr, hr * R.u, hr * R.v};
      const double uxs = vr * tx + us * ty;
      const double vys = vr * nx + us * ny;
      const double X = hr * A, Y = ar - us;
      const double hs = SWE_DIV(X, Y);
      const double Us[3] = {hs, hs * uxs, hs * vys};
      const double sp = smax(0., ar);
      double lsp = 0., lUr[3], lUs[3];
      for (int q = 0; q < 3; ++q) {
        lsp += lF[q] * (Us[q] - Ur[q]);
        lUs[q] = sp * lF[q];
        lUr[q] = -sp * lF[q];
      }
      if (dlt(0., ar)) lar += lsp;
      elem_flux_rev(nx, ny, Ur[0], Ur[1], Ur[2], lF, &lUr[0], &lUr[1], &lUr[2]);
      const double lhs = lUs[0] + lUs[1] * uxs + lUs[2] * vys;
      const double luxs = lUs[1] * hs, lvys = lUs[2] * hs;
      const double lX = SWE_DIV(lhs, Y), lY = -SWE_DIV(lhs * hs, Y);
      lhr += lX * A;
      lA += lX * hr;
      lar += lY;
      lus -= lY;
      lvr += luxs * tx + lvys * nx;
      lus += luxs * ty + lvys * ny;
      lhr += lUr[0] + lUr[1] * R.u + lUr[2] * R.v;
      lRu += lUr[1] * hr;
      lRv += lUr[2] * hr;
    } else {
      const double Ul[3] = {hl, hl * L.u, hl * L.v};
      const double uxs = vl * tx + us * ty;
      const double vys = vl * nx + us * ny;
      const double X = hl * B, Y = al - us;
      const double hs = SWE_DIV(X, Y);
      const double Us[3] = {hs, hs * uxs, hs * vys};
      const double sm = smin(0., al);
      double lsm = 0., lUl[3], lUs[3];
      for (int q = 0; q < 3; ++q) {
        lsm += lF[q] * (Us[q] - Ul[q]);
        lUs[q] = sm * lF[q];
        lUl[q] = -sm * lF[q];
      }
      if (dlt(al, 0.)) lal += lsm;
      elem_flux_rev(nx, ny, Ul[0], Ul[1], Ul[2], lF, &lUl[0], &lUl[1], &lUl[2]);
      const double lhs = lUs[0] + lUs[1] * uxs + lUs[2] * vys;
      const double luxs = lUs[1] * hs, lvys = lUs[2] * hs;
      const double lX = SWE_DIV(lhs, Y), lY = -SWE_DIV(lhs * hs, Y);
      lhl += lX * B;
      lB += lX * hl;
      lal += lY;
      lus -= lY;
      lvl += luxs * tx + lvys * nx;
      lus += luxs * ty + lvys * ny;
      lhl += lUl[0] + lUl[1] * L.u + lUl[2] * L.v;
      lLu += lUl[1] * hl;
      lLv += lUl[2] * hl;
    }
    // us = N / D
    const double lN = SWE_DIV(lus, D);
    const double lD = -SWE_DIV(lus * us, D);
    lhr += lD * A;
    lA += lD * hr;
    lhl -= lD * B;
    lB -= lD * hl;
    lA += lN * hr * ur;
    lhr += lN * A * ur;
    lur += lN * A * hr;
    lB -= lN * hl * ul;
    lhl -= lN * B * ul;
    lul -= lN * B * hl;
    lhl += lN * hl;
    lhr -= lN * hr;
    lar += lA;
    lur -= lA;
    lal += lB;
    lul -= lB;
    wavespeeds_rev(ws, ul, hl, ur, hr, lal, lar, &lul, &lhl, &lur, &lhr);
  }
  lLu += lul * nx + lvl * tx;
  lLv += lul * ny + lvl * ty;
  lRu += lur * nx + lvr * tx;
  lRv += lur * ny + lvr * ty;
  lL[0] += lhl;
  lL[1] += lLu;
  lL[2] += lLv;
  lR[0] += lhr;
  lR[1] += lRu;
  lR[2] += lRv;
  *lb -= lhl + lhr;
}

}  // namespace swe
