// swe_adjoint.cu -- discrete adjoint of the Runge-Kutta step.
//
// The reverse of one stage (forward: k_recon1/k_recon2 -> k_flux -> k_drain ->
// k_update, src/SpaceDisc.cpp:33-74, src/TimeDisc.cpp:3-66,
// src/Solvers.cpp:5-59) is four kernels, each a gather so that only the rare
// PartWet2 node-maximum scatter and the bathymetry gradient use atomics:
//   R1 k_adj_update  cell   RHS + Shu-Osher + ConsAssigner reverse; per slot:
//                           flux adjoint, draining-dt adjoint and its route
//   R2 k_adj_drain   cell   gathers the draining-dt adjoint (own slots and the
//                           neighbours' twin slots), reverses the draining dt
//   R3 k_adj_flux    edge   gathers both slots' flux adjoints; flux plugin
//                           reverse by a forward-mode Jacobian (Dual<7>)
//   R4 k_adj_recon   cell   reconstruction reverse: interface values and
//                           source gradients to the cell state; bathymetry
//                           adjoints straight to node z
// The forward intermediates of the stage (interface slots, fluxes, draining
// time steps, node maxima) are recomputed from the stage input right before
// its reverse.  dt is the forward's, frozen: the CFL ratio's dependence on the
// state is not differentiated.
#include <cuda_runtime.h>

#include <algorithm>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "swe_adjoint.cuh"
#include "swe_dual.cuh"
#include "swe_flux_adjoint.cuh"

namespace swe {

namespace {

constexpr double kInfA = __builtin_huge_val();

// draining time step of the stage (k_drain without the pass reset, so the
// pass-1 node maxima stay available to the reverse)
__global__ void __launch_bounds__(256) k_drain_keep(DevMesh m, DevWork wk, const double* __restrict__ W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.C) return;
  const double h = W[i] - m.bc[i];
  double d;
  if (!is_wet(h)) {
    d = 0.;
  } else {
    const unsigned own = m.cown[i];
    double sum = 0.;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double f = wk.f0[gidx(m, m.cedge[k * m.C + i], m.E)];
      sum += smax(0., ((own >> k) & 1u) ? f : -f);
    }
    d = dgtc(sum, kTol) ? SWE_DIV(m.area[i] * h, sum) : kInfA;
  }
  wk.drain[i] = d;
}

__global__ void k_fold_scatter(int C, double* lamp, double* lscatter) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < C) {
    lamp[i] += lscatter[i];
    lscatter[i] = 0.;
  }
}

__global__ void k_gather_gauges(const double* W, const int* g, int n, double* out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) out[q] = W[g[q]];
}

// out = a + b (3C arrays)
__global__ void k_add3(int C, const double* a, const double* b, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < C) {
    out[i] = a[i] + b[i];
    out[C + i] = a[C + i] + b[C + i];
    out[2 * C + i] = a[2 * C + i] + b[2 * C + i];
  }
}

// the gauge seeds of step n = *s0 + loc, when it ends an observation window
__global__ void k_seed_gauges_seg(double* lamw, const int* g, int n_g, const double* tg, const long long* s0,
                                  long long loc, long long obs) {
  const long long n = *s0 + loc;
  if ((n + 1) % obs != 0) return;
  const long long j = (n + 1) / obs - 1;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n_g) atomicAdd(lamw + g[q], tg[j * n_g + q]);
}

// dst[q] = dts[(*s0 + loc) I + q]: the recorded dts (one per instance) of a
// step of the current segment
__global__ void k_fetch_dt(double* dst, const double* dts, const long long* s0, long long loc, int n_inst) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n_inst) dst[q] = dts[(*s0 + loc) * n_inst + q];
}
__global__ void k_set_i64(long long* dst, long long v) {
  if (threadIdx.x == 0) *dst = v;
}

// ---------------------------------------------------------------- R1: update
// nst: the stage's conservative state before ConsAssigner ([3][C], kept by the
// segment recompute), or null to recompute it from the stage's fluxes.
__global__ void __launch_bounds__(256, 4) k_adj_update(DevMesh m, DevWork wk, AdjWork aw, const double* Wp,
                                                    const double* Up, const double* Vp, const double* W0,
                                                    const double* U0, const double* V0, const double* nst, Stage st,
                                                    int batched) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.C) return;
  const int C = m.C;
  const int inst = batched ? m.cinst[i] : 0;
  const double dt = st.first ? wk.dt[inst] : st.c * wk.dt[inst];
  const unsigned own = m.cown[i];
  const double dti = wk.drain[i];
  const double b = m.bc[i];
  // ---- draining-limited step of each local edge (as the forward selected it)
  double dtk_[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int slot = k * C + i;
    const double F0 = wk.f0[gidx(m, m.cedge[slot], m.E)];
    const int nb = m.cnbr[slot];
    const double dtik = nb < 0 ? kInfA : wk.drain[gidx(m, nb, C)];
    dtk_[k] = dgt0(((own >> k) & 1u) ? F0 : -F0) ? smin(dt, dti) : smin(dt, dtik);
  }
  const double h0 = W0[i] - b;
  const double hp = st.first ? 0. : Wp[i] - b;
  double n0, n1, n2;
  if (nst) {
    n0 = nst[i];
    n1 = nst[C + i];
    n2 = nst[2 * C + i];
  } else {
    // forward recompute of the RHS accumulation and the combination
    double r0 = 0., r1 = 0., r2 = 0.;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int slot = k * C + i;
      const int e = m.cedge[slot];
      const double sgn = ((own >> k) & 1u) ? 1. : -1.;
      const double F0 = wk.f0[e], F1 = wk.f1[e], F2 = wk.f2[e];
      const double dtk = dtk_[k];
      const double c_ek = m.cek[slot];
      const double h_ek = wk.ew[slot] - m.ze[slot];
      const double s = dtk * sgn * c_ek;
      r0 -= s * F0;
      r1 -= s * F1;
      r2 -= s * F2;
      const double q = dt * (1. / 3.);
      r1 -= q * wk.sx[slot] * h_ek;
      r2 -= q * wk.sy[slot] * h_ek;
      const double p = 0.5 * h_ek * h_ek;
      r1 += dtk * (m.cnxc[slot] * p);
      r2 += dtk * (m.cnyc[slot] * p);
    }
    const double c00 = h0, c01 = h0 * U0[i], c02 = h0 * V0[i];
    if (st.first) {
      n0 = c00 + r0;
      n1 = c01 + r1;
      n2 = c02 + r2;
    } else {
      const double c11 = hp * Up[i], c12 = hp * Vp[i];
      n0 = st.a * c00 + st.b * hp + r0;
      n1 = st.a * c01 + st.b * c11 + r1;
      n2 = st.a * c02 + st.b * c12 + r2;
    }
  }
  // ---- reverse of ConsAssigner (src/Assigners.cpp:28-44)
  const double lw = aw.lam[i], lu = aw.lam[C + i], lv = aw.lam[2 * C + i];
  double lbc = 0., ln0 = 0., ln1 = 0., ln2 = 0.;
  if (!is_wet(n0)) {
    lbc += lw;
  } else {
    double ih, dih;
    if (dltc(n0, kEta1)) {
      const double n2_ = n0 * n0;
      const double h4 = fma(n2_, n2_, kEta4);
      const double sq = SWE_SQRT(h4);
      ih = kSqrt2 * n0 * SWE_DIV(1., sq);
      dih = kSqrt2 * fma(-n2_, n2_, kEta4) * SWE_DIV(1., h4 * sq);
    } else {
      ih = SWE_DIV(1., n0);
      dih = -ih * ih;
    }
    lbc += lw;
    ln0 = fma(fma(lu, n1, lv * n2), dih, lw);
    ln1 = lu * ih;
    ln2 = lv * ih;
  }
  // ---- combination
  const double a0c = st.first ? 1. : st.a;
  const double lc00 = a0c * ln0, lc01 = a0c * ln1, lc02 = a0c * ln2;
  {
    const double lh0 = fma(lc01, U0[i], fma(lc02, V0[i], lc00));
    aw.lam0[i] += lh0;
    aw.lam0[C + i] = fma(lc01, h0, aw.lam0[C + i]);
    aw.lam0[2 * C + i] = fma(lc02, h0, aw.lam0[2 * C + i]);
    lbc -= lh0;
  }
  if (!st.first) {
    const double lc10 = st.b * ln0, lc11 = st.b * ln1, lc12 = st.b * ln2;
    const double lhp = fma(lc11, Up[i], fma(lc12, Vp[i], lc10));
    aw.lamp[i] += lhp;
    aw.lamp[C + i] = fma(lc11, hp, aw.lamp[C + i]);
    aw.lamp[2 * C + i] = fma(lc12, hp, aw.lamp[2 * C + i]);
    lbc -= lhp;
  }
  // ---- reverse of the RHS (src/TimeDisc.cpp:21-36), per local edge
  const double q = dt * (1. / 3.);
  const double ln1q = ln1 * q, ln2q = ln2 * q;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int slot = k * C + i;
    const int e = gidx(m, m.cedge[slot], m.E);
    const bool out = (own >> k) & 1u;
    const double F0 = wk.f0[e], F1 = wk.f1[e], F2 = wk.f2[e];
    const double c_ek = m.cek[slot];
    const double h_ek = wk.ew[slot] - m.ze[slot];
    const double p = 0.5 * h_ek * h_ek;
    const double dtk = dtk_[k];
    const double sc = out ? c_ek : -c_ek;  // sgn c_ek
    const double s = dtk * sc;
    const double nxc = m.cnxc[slot], nyc = m.cnyc[slot];
    const double lpn = fma(ln1, nxc, ln2 * nyc);
    const double ls = -fma(ln0, F0, fma(ln1, F1, ln2 * F2));
    const double ldtk = fma(ls, sc, lpn * p);
    const double lh = fma(dtk * lpn, h_ek, -fma(ln1q, wk.sx[slot], ln2q * wk.sy[slot]));
    aw.lsx[slot] = -ln1q * h_ek;
    aw.lsy[slot] = -ln2q * h_ek;
    aw.lF0[slot] = -ln0 * s;
    aw.lF1[slot] = -ln1 * s;
    aw.lF2[slot] = -ln2 * s;
    aw.lew[slot] = lh;
    aw.leu[slot] = 0.;
    aw.lev[slot] = 0.;
    aw.lze[slot] = -lh;
    // route of the draining time step actually selected by min(dt, .)
    const int nb = m.cnbr[slot];
    int route = 0;
    if (dgt0(out ? F0 : -F0)) {
      if (dlt(dti, dt)) route = 1;
    } else if (nb >= 0) {
      if (dlt(wk.drain[gidx(m, nb, C)], dt)) route = 2;
    }
    aw.ldtk[slot] = route ? ldtk : 0.;
    aw.route[slot] = (unsigned char)route;
  }
  aw.lbc[i] = lbc;
}

// ---------------------------------------------------------------- R2: drain
__global__ void __launch_bounds__(256) k_adj_drain(DevMesh m, DevWork wk, AdjWork aw, const double* Wp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.C) return;
  const int C = m.C;
  double ld = 0.;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int slot = k * C + i;
    if (aw.route[slot] == 1) ld += aw.ldtk[slot];
    const int tw = aw.twin[slot];
    if (tw >= 0) {
      const int t2 = gidx(m, tw, 3 * C);
      if (aw.route[t2] == 2) ld += aw.ldtk[t2];
    }
  }
  const double h = Wp[i] - m.bc[i];
#pragma unroll
  for (int k = 0; k < 3; ++k) aw.lF0d[k * C + i] = 0.;
  if (ld == 0. || !is_wet(h)) return;
  const unsigned own = m.cown[i];
  double sum = 0.;
  double fk[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double f = wk.f0[gidx(m, m.cedge[k * C + i], m.E)];
    fk[k] = ((own >> k) & 1u) ? f : -f;
    sum += smax(0., fk[k]);
  }
  if (!dgtc(sum, kTol)) return;
  const double A = m.area[i];
  const double d = SWE_DIV(A * h, sum);
  const double lAh = SWE_DIV(ld, sum);
  const double ls = -SWE_DIV(ld * d, sum);
  const double lh = lAh * A;
  aw.lamp[i] += lh;
  aw.lbc[i] -= lh;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (dlt(0., fk[k])) aw.lF0d[k * C + i] = ((own >> k) & 1u) ? ls : -ls;
  }
}

// ---------------------------------------------------------------- R3: flux
template <int FLUX, int WS>
__global__ void __launch_bounds__(256, 4) k_adj_flux(DevMesh m, DevWork wk, AdjWork aw, const double* Wp) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m.E) return;
  const int o = gidx(m, m.eown[e], m.C), nb = m.enb[e];
  const int sl = gidx(m, m.eslotl[e], 3 * m.C);
  double lF[3] = {aw.lF0[sl] + aw.lF0d[sl], aw.lF1[sl], aw.lF2[sl]};
  const double nx = m.enx[e], ny = m.eny[e];
  if (nb < 0) {
    // wall: F = ElemFlux(n, (h_owner, 0, 0)) -> dF/dh = (0, h nx, h ny)
    const double h = Wp[o] - m.bc[o];
    aw.lhwall[sl] = is_wet(h) ? (lF[1] * nx + lF[2] * ny) * h : 0.;
    return;
  }
  aw.lhwall[sl] = 0.;
  const int sr = gidx(m, m.eslotr[e], 3 * m.C);
  lF[0] += aw.lF0[sr] + aw.lF0d[sr];
  lF[1] += aw.lF1[sr];
  lF[2] += aw.lF2[sr];
  if (lF[0] == 0. && lF[1] == 0. && lF[2] == 0.) return;
  EdgeGeom g;
  g.nx = nx;
  g.ny = ny;
  g.tx = m.etx[e];
  g.ty = m.ety[e];
  g.b = m.ezm[e];
  g.lmin = m.elmin[e];
  SideState L{wk.ew[sl], wk.eu[sl], wk.ev[sl]};
  SideState R{wk.ew[sr], wk.eu[sr], wk.ev[sr]};
  double lL[3] = {0., 0., 0.}, lR[3] = {0., 0., 0.}, lb = 0.;
  flux_reverse(FLUX, WS, g, L, R, lF, lL, lR, &lb, wk.ftape, m.E, e);
  aw.lew[sl] += lL[0];
  aw.leu[sl] += lL[1];
  aw.lev[sl] += lL[2];
  aw.lew[sr] += lR[0];
  aw.leu[sr] += lR[1];
  aw.lev[sr] += lR[2];
  aw.lze[sl] += lb;
}

// ------------------------------------------------------- R4: reconstruction
// Pass-1 reconstruction of cell c restated for the reverse: type 0 dry,
// 1 partially wet (PartWet1 level in w0), 2 fully wet; for fully wet: the
// combination mask and whether the plane survived positivity and the limiter.
struct P1 {
  int type, mask;
  bool kept;
  double w0;
};
__device__ P1 pass1(const DevWork& wk, const double* W, int c) {
  // the class the forward pass 1 stored; the level of a partially-wet cell is
  // its PartWet1 level, of a fully-wet cell its own w
  const unsigned cl = wk.cls[c];
  P1 r{(int)(cl & 3u), (int)((cl >> 2) & 7u), ((cl >> 5) & 1u) != 0u, 0.};
  if (r.type == 1) r.w0 = wk.pwrec[c];
  else if (r.type == 2) r.w0 = W[c];
  return r;
}

// Pass-1 value of cell c at its local node kn (AtPoint(P).w), and where its
// derivative goes: dstate = d value / d W[c]; static part to node z.
__device__ double pass1_node_value(const DevMesh& m, const DevWork& wk, const double* W, int c, int kn) {
  const int C = m.C;
  const double z = m.zn[kn * C + c];
  const P1 p = pass1(wk, W, c);
  if (p.type == 0) return m.dry[(size_t)c * kDryStride + kn];
  double off = 0.;
  if (p.type == 2 && p.kept) off = m.combo[combo_off(m.C, c, p.mask) + 8 + kn];
  const double a = p.w0 + off;
  return dge0(a - z) ? a : z;
}

// node id of local node k of cell c
__device__ __forceinline__ int cnode(const DevMesh& m, int c, int k) { return gidx(m, m.cnode[k * m.C + c], m.N); }

// adds l to the node-z gradient through the edge-centre bathymetry of slot
// (c, k): the midpoint of the edge's two nodes
__device__ __forceinline__ void lam_edge_z(const DevMesh& m, AdjWork& aw, int c, int k, double l) {
  if (l == 0.) return;
  const int e = gidx(m, m.cedge[k * m.C + c], m.E);
  atomicAdd(aw.lz + gidx(m, aw.edge_nodes[2 * e], m.N), 0.5 * l);
  atomicAdd(aw.lz + gidx(m, aw.edge_nodes[2 * e + 1], m.N), 0.5 * l);
}
// ... through the centroid bathymetry of cell c
__device__ __forceinline__ void lam_cell_z(const DevMesh& m, AdjWork& aw, int c, double l) {
  if (l == 0.) return;
  const double k3 = 1. / 3.;
  for (int k = 0; k < 3; ++k) atomicAdd(aw.lz + cnode(m, c, k), k3 * l);
}

// PartWet1 level and its derivatives with respect to (w, z0, z1, z2) of the
// cell (src/MUSCLObject.cpp:86-112), recomputed from the node bathymetry.
template <class T>
__device__ T partwet1_t(const T& w, const T& z0, const T& z1, const T& z2, double root) {
  const double k3 = 1. / 3.;
  T bc = z0 * k3 + z1 * k3 + z2 * k3;
  T h = w - bc;
  T b13 = z0, b23 = z0;
  if (dlt(val(b13), val(z1))) b13 = z1;
  if (dlt(val(b13), val(z2))) b13 = z2;
  if (dlt(val(z1), val(b23))) b23 = z1;
  if (dlt(val(z2), val(b23))) b23 = z2;
  T b12 = 3. * bc - b23 - b13;
  T bdel = b12 + (1. / 3.) * (b13 - b12) * (b13 - b12) / (b13 - b23);
  if (dle(val(b13), val(w))) return w;
  if (dle(val(w), val(bdel))) return b23 + tcbrt(3. * h * (b13 - b23) * (b12 - b23));
  T a = -3. * b13;
  T bb = 3. * (b12 * b13 + b13 * b23 - b12 * b23);
  T cc = (b13 - b23) * (3. * h * (b13 - b12) - b12 * (b12 + b23)) - b23 * b23 * b13;
  // root: the level the forward pass found (the same cubic's root)
  if (dle(val(b12), root) && dle(root, val(b13))) return bisection_root_t(cc, bb, a, val(b12), val(b13), root);
  return bisection_t(cc, bb, a, val(b12), val(b13));
}

// PartWet2 (src/MUSCLObject.cpp:114-191) recomputed from the sorted vertices
// with dual (w, w23, z_lo, z_mid, z_hi): level at the centroid and slope.
// Returns false if it falls back to PartWet1.
template <class T>
__device__ bool partwet2_t(const Pw2Rec& r, const T& w, const T& w23, const T& zl, const T& zm, const T& zh,
                           const T& bc, T* w0, T* gx, T* gy) {
  T b23 = zl, b12 = zm, b13 = zh;
  if (dlt(val(b13), val(w)) || r.flat) return false;
  T h23 = w23 - b23;
  T ratio_b = (b12 - b23) / (b13 - b23);
  T h_delim1 = 1. / 3. * h23 * ratio_b;
  T h_delim2 = 1. / 3. * h23 * (2. * b13 - b12 - b23) / (b13 - b23);
  T hi = w - bc;
  T ratio_h = hi / h23;
  const T P0x(r.p[0][0]), P0y(r.p[0][1]), P1x(r.p[1][0]), P1y(r.p[1][1]), P2x(r.p[2][0]), P2y(r.p[2][1]);
  T p1x, p1y, p1z, p2x, p2y, p2z;
  if (dle(val(hi), val(h_delim1))) {
    T k2 = tsqrt(3. * ratio_h / ratio_b);
    p1x = k2 * P1x + (1. - k2) * P0x;
    p1y = k2 * P1y + (1. - k2) * P0y;
    p1z = k2 * zm + (1. - k2) * zl;
    T k3 = tsqrt(3. * ratio_h * ratio_b);
    p2x = k3 * P2x + (1. - k3) * P0x;
    p2y = k3 * P2y + (1. - k3) * P0y;
    p2z = k3 * zh + (1. - k3) * zl;
  } else if (dle(val(h_delim2), val(hi))) {
    T delta_w = 1.5 * (hi - h_delim2);
    p1x = P1x; p1y = P1y; p1z = zm;
    p2x = P2x; p2y = P2y; p2z = zh;
    p2z = p2z + delta_w;
  } else {
    T alpha = 3. * ratio_h;
    T beta = (b13 - b12) / (b13 - b23);
    T k1 = 1. - bisection_t((1. + beta - alpha) / (beta * beta), (alpha - 3.) / beta, T(0.), 0., 1.);
    if (dltc(val(k1), kTol)) return false;
    T bp1 = k1 * b13 + (1. - k1) * b12;
    p1x = P1x; p1y = P1y; p1z = zm;
    p2x = k1 * P2x + (1. - k1) * P1x;
    p2y = k1 * P2y + (1. - k1) * P1y;
    p2z = bp1;
  }
  plane_gradient_t(P0x, P0y, zl, p1x, p1y, p1z, p2x, p2y, p2z, gx, gy);
  *w0 = w23 + (*gx * r.tp0x + *gy * r.tp0y);
  return true;
}

// reverse of one interface slot write (src/SpaceDisc.cpp:24-29): given the
// adjoints of the slot (w, u, v, sx, sy) and the forward inputs of AtPoint,
// returns adjoints of (w0 + off) [law], u0, v0, gx, gy, and of the slot's
// edge bathymetry (ze).
template <bool COR0>
__device__ void slot_reverse(double ze, double a_w, double u0, double v0, double cor, double lw, double lu, double lv,
                             double lsx, double lsy, double* law, double* lu0, double* lv0, double* lgx, double* lgy,
                             double* lze) {
  *lgx = lsx;
  *lgy = lsy;
  // AtPoint dry check
  double aw_ = a_w, au = u0, av = v0;
  const bool wet_at = dge0(a_w - ze);
  if (!wet_at) {
    aw_ = ze;
    au = 0.;
    av = 0.;
  }
  // src += cor (-v, u) uses the assigned velocities
  double lue = lu, lve = lv;
  if (!COR0) {
    lue = fma(cor, lsy, lu);
    lve = fma(-cor, lsx, lv);
  }
  double law_ = 0., lau = 0., lav = 0., lz = 0.;
  const double h = aw_ - ze;
  if (!is_wet(h)) {
    lz += lw;
  } else {
    law_ = lw;
    if (dltc(h, kEta1)) {
      const double t = h * h + kEta2;
      const double st = SWE_SQRT(t);
      const double s = SWE_DIV(kSqrt2 * h, st);
      const double ds = SWE_DIV(kSqrt2 * kEta2, t * st);
      lau = lue * s;
      lav = lve * s;
      const double lh = (lue * au + lve * av) * ds;
      law_ += lh;
      lz -= lh;
    } else {
      lau = lue;
      lav = lve;
    }
  }
  if (wet_at) {
    *law = law_;
    *lu0 = lau;
    *lv0 = lav;
  } else {
    *law = 0.;
    *lu0 = 0.;
    *lv0 = 0.;
    lz += law_;
  }
  *lze = lz;
}

// Adjoint of the z of the three points of a plane slope (plane_gradient):
// with M = [[x1-x0, y1-y0], [x2-x0, y2-y0]] the slope is M^-1 (z1-z0, z2-z0),
// so (lz1, lz2) = M^-T (lg0, lg1) and lz0 = -(lz1 + lz2).
__device__ void plane_points_adjoint(const double* px, const double* py, double lg0, double lg1, double* lp) {
  const double a00 = px[1] - px[0], a01 = py[1] - py[0];
  const double a10 = px[2] - px[0], a11 = py[2] - py[0];
  const double det = a00 * a11 - a01 * a10;
  const double l1 = SWE_DIV(lg0 * a11 - lg1 * a10, det);
  const double l2 = SWE_DIV(-lg0 * a01 + lg1 * a00, det);
  lp[0] = -(l1 + l2);
  lp[1] = l1;
  lp[2] = l2;
}
// points of the fully-wet plane of cell c for neighbour combination `mask`
// (neighbour centroid, or edge centre where the neighbour is partially wet),
// relative to c's centroid
__device__ void combo_plane_points(const DevMesh& m, int c, int mask, double* px, double* py) {
  const int C = m.C;
  const Pw2Rec& r = m.pw2[c];
  for (int k = 0; k < 3; ++k) {
    if ((mask >> k) & 1) {
      px[k] = r.dedge[k][0];
      py[k] = r.dedge[k][1];
    } else {
      const Pw2Rec& rn = m.pw2[gidx(m, m.cnbr[k * C + c], C)];
      px[k] = (rn.p[0][0] + rn.tp0x) - (r.p[0][0] + r.tp0x);
      py[k] = (rn.p[0][1] + rn.tp0y) - (r.p[0][1] + r.tp0y);
    }
  }
}
// adjoint lp[k] of the plane's point z -> node bathymetry
__device__ void combo_points_to_nodes(const DevMesh& m, AdjWork& aw, int c, int mask, const double* lp) {
  for (int k = 0; k < 3; ++k) {
    if (lp[k] == 0.) continue;
    if ((mask >> k) & 1) lam_edge_z(m, aw, c, k, lp[k]);
    else lam_cell_z(m, aw, gidx(m, m.cnbr[k * m.C + c], m.C), lp[k]);
  }
}

// the plane-point adjoint table of every cell and neighbour combination
__global__ void k_plane_adj_init(DevMesh m, double* padj) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m.C) return;
  double* out = padj + (size_t)c * 48;
  bool interior = true;
  for (int k = 0; k < 3; ++k) interior = interior && m.cnbr[k * m.C + c] >= 0;
  for (int q = 0; q < 8; ++q) {
    double lx[3] = {0., 0., 0.}, ly[3] = {0., 0., 0.};
    if (interior) {
      double px[3], py[3];
      combo_plane_points(m, c, q, px, py);
      plane_points_adjoint(px, py, 1., 0., lx);
      plane_points_adjoint(px, py, 0., 1., ly);
    }
    for (int k = 0; k < 3; ++k) {
      out[q * 6 + k] = lx[k];
      out[q * 6 + 3 + k] = ly[k];
    }
  }
}

// Forward-only part of a partially-wet cell's reverse: the PartWet2 plane (or
// PartWet1 level) with its derivatives, and where the PartWet2 node maximum
// w23 came from.  It reads no adjoint, so it runs beside R1-R3.
__device__ void pw_jacobian(const DevMesh& m, const DevWork& wk, const AdjWork& aw, const double* W, int i,
                            PwJac* out) {
  const int C = m.C;
  const double w = W[i];
  const Pw2Rec& r = m.pw2[i];
  const double w23 = order_val(wk.maxwp[gidx(m, r.lo, m.N)]);
  typedef Dual<5> D5;  // PartWet2 over (w, w23, z_lo, z_mid, z_hi)
  D5 zc[3];
  for (int k = 0; k < 3; ++k) zc[k] = D5(m.zn[k * C + i]);
  const D5 zl = D5::var(r.p[0][2], 2), zm = D5::var(r.p[1][2], 3), zh = D5::var(r.p[2][2], 4);
  for (int s = 0; s < 3; ++s) zc[r.sk[s]] = (s == 0) ? zl : (s == 1 ? zm : zh);
  const double k3 = 1. / 3.;
  D5 bcd = zc[0] * k3 + zc[1] * k3 + zc[2] * k3;
  bcd.v = m.bc[i];  // the forward's centroid bathymetry
  D5 w0D, gxD, gyD;
  PwJac J;
  J.plane = partwet2_t(r, D5::var(w, 0), D5::var(w23, 1), zl, zm, zh, bcd, &w0D, &gxD, &gyD) ? 1 : 0;
  J.route = 0;
  J.target = r.lo;
  J.mask = -1;
  for (int q = 0; q < 4; ++q) J.rc[q] = 0.;
  if (!J.plane) {
    // PartWet1 level: dual over (w, z0, z1, z2)
    typedef Dual<4> D;
    const double lvl = wk.pwrec[i];
    const D y = partwet1_t(D::var(w, 0), D::var(m.zn[i], 1), D::var(m.zn[C + i], 2), D::var(m.zn[2 * C + i], 3), lvl);
    J.w0 = lvl;
    J.gx = 0.;
    J.gy = 0.;
    for (int q = 0; q < 5; ++q) {
      J.jw0[q] = q < 4 ? y.d[q] : 0.;
      J.jgx[q] = 0.;
      J.jgy[q] = 0.;
    }
    *out = J;
    return;
  }
  J.w0 = w0D.v;
  J.gx = gxD.v;
  J.gy = gyD.v;
  for (int q = 0; q < 5; ++q) {
    J.jw0[q] = w0D.d[q];
    J.jgx[q] = gxD.d[q];
    J.jgy[q] = gyD.d[q];
  }
  // w23 = max over the cells around the lowest node of their pass-1 value
  const int nd = gidx(m, r.lo, m.N);
  int best = -1, bestk = 0;
  for (int q = aw.node_ptr[nd]; q < aw.node_ptr[nd + 1]; ++q) {
    const int cq = aw.node_cells[gidx(m, q, 3 * C)];
    const int c = gidx(m, cq >> 2, C), kn = cq & 3;
    if (pass1_node_value(m, wk, W, c, kn) == w23) {
      best = c;
      bestk = kn;
      break;
    }
  }
  if (best >= 0) {
    const P1 pc = pass1(wk, W, best);
    const double zc_ = m.zn[bestk * C + best];
    J.route = 0;
    J.target = cnode(m, best, bestk);
    if (pc.type == 0) {
      // dry plane value at the node: a function of bathymetry only
      typedef Dual<3> E;
      const Pw2Rec& rb = m.pw2[best];
      E z0 = E::var(m.zn[best], 0), z1 = E::var(m.zn[C + best], 1), z2 = E::var(m.zn[2 * C + best], 2);
      E sxd, syd;
      plane_gradient_t(E(rb.dnode[0][0]), E(rb.dnode[0][1]), z0, E(rb.dnode[1][0]), E(rb.dnode[1][1]), z1,
                       E(rb.dnode[2][0]), E(rb.dnode[2][1]), z2, &sxd, &syd);
      E bcb = z0 * k3 + z1 * k3 + z2 * k3;
      E a = bcb + (sxd * rb.dnode[bestk][0] + syd * rb.dnode[bestk][1]);
      if (dge0(a.v - zc_)) {
        J.route = 1;
        J.target = best;
        for (int q = 0; q < 3; ++q) J.rc[q] = a.d[q];
      }
    } else {
      double off_n = 0.;
      if (pc.type == 2 && pc.kept) off_n = m.combo[combo_off(m.C, best, pc.mask) + 8 + bestk];
      if (dge0((pc.w0 + off_n) - zc_)) {
        J.target = best;
        if (pc.type == 2) {
          // the fully-wet cell's level, and its vertex offset a_k = g . (P_k - T)
          // moving with the plane's point z
          J.route = 2;
          if (pc.kept) {
            const Pw2Rec& rb = m.pw2[best];
            const double* T = aw.padj + (size_t)best * 48 + pc.mask * 6;
            const double dx = rb.dnode[bestk][0], dy = rb.dnode[bestk][1];
            for (int k = 0; k < 3; ++k) J.rc[k] = fma(dx, T[k], dy * T[3 + k]);
            J.mask = pc.mask;
          }
        } else {
          typedef Dual<4> F4;
          const F4 y = partwet1_t(F4::var(W[best], 0), F4::var(m.zn[best], 1), F4::var(m.zn[C + best], 2),
                                  F4::var(m.zn[2 * C + best], 3), pc.w0);
          J.route = 3;
          for (int q = 0; q < 4; ++q) J.rc[q] = y.d[q];
          // Regularised at the wetting front: the level is b23 + cbrt(3 h K)
          // for small depth h, whose slope in w grows like h^(-2/3); fed back
          // through PartWet2 it made the reverse grow geometrically (1e24
          // after 500 steps on beds whose bumps emerge) while finite
          // differences of the forward stay ~1e-5.  Below the reference's
          // desingularisation depth kEta1 the w-slope is taken at h = kEta1
          // (scaled by (h / kEta1)^(2/3)).
          const double hb = W[best] - m.bc[best];
          const double rd = aw.reg_depth;
          if (rd > 0. && dltc(hb, rd)) J.rc[0] *= dge0(hb) ? cbrt(SWE_DIV(hb * hb, rd * rd)) : 0.;
        }
      }
    }
  }
  *out = J;
}

// Reverse of the reconstruction of cell i; partially-wet cells contract the
// Jacobians pw_jacobian stored for them.
template <bool COR0>
__device__ void adj_recon_cell(const DevMesh& m, const DevWork& wk, AdjWork aw, const double* W, const double* U,
                               const double* V, int i, int batched) {
  const int C = m.C;
  const int inst = batched ? m.cinst[i] : 0;
  const double cor = m.inst_cor[inst];
  const double w = W[i], u = U[i], v = V[i];
  double lw_i = 0., lu_i = 0., lv_i = 0.;
  double lbc = aw.lbc[i];
  // wall-flux depth adjoints of the owned wall edges
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double lh = aw.lhwall[k * C + i];
    if (lh != 0. && m.cnbr[k * C + i] < 0 && ((m.cown[i] >> k) & 1u)) {
      lw_i += lh;
      lbc -= lh;
    }
  }
  const P1 p = pass1(wk, W, i);
  if (p.type == 0) {
    const double* dr = m.dry + (size_t)i * kDryStride;
    // interface values (dew_k, 0, 0) and slope (sx, sy) are functions of the
    // cell's node z: dual over z0..z2
    typedef Dual<3> D;
    D z0 = D::var(m.zn[i], 0), z1 = D::var(m.zn[C + i], 1), z2 = D::var(m.zn[2 * C + i], 2);
    const Pw2Rec& r = m.pw2[i];
    // node positions relative to the centroid (slopes depend on differences only)
    D sxd, syd;
    plane_gradient_t(D(r.dnode[0][0]), D(r.dnode[0][1]), z0, D(r.dnode[1][0]), D(r.dnode[1][1]), z1,
                     D(r.dnode[2][0]), D(r.dnode[2][1]), z2, &sxd, &syd);
    const double k3 = 1. / 3.;
    const D bcd = z0 * k3 + z1 * k3 + z2 * k3;
    double lz3[3] = {0., 0., 0.};
    for (int k = 0; k < 3; ++k) {
      const int slot = k * C + i;
      double law, lu0, lv0, lgx, lgy, lze;
      slot_reverse<COR0>(m.ze[slot], dr[3 + k], 0., 0., cor, aw.lew[slot], aw.leu[slot], aw.lev[slot], aw.lsx[slot],
                   aw.lsy[slot], &law, &lu0, &lv0, &lgx, &lgy, &lze);
      const D e0v = bcd + (sxd * r.dedge[k][0] + syd * r.dedge[k][1]);
      for (int q = 0; q < 3; ++q) lz3[q] = fma(law, e0v.d[q], fma(lgx, sxd.d[q], fma(lgy, syd.d[q], lz3[q])));
      lam_edge_z(m, aw, i, k, lze + aw.lze[slot]);
    }
    for (int q = 0; q < 3; ++q)
      if (lz3[q] != 0.) atomicAdd(aw.lz + cnode(m, i, q), lz3[q]);
    lam_cell_z(m, aw, i, lbc);
    return;
  }
  // forward description of the final interface values: level w0 + off_k, velocity, slope
  double w0 = w, gx = 0., gy = 0., off[3] = {0., 0., 0.};
  const PwJac* J = nullptr;
  if (p.type == 2) {
    if (p.kept) {
      const double* rec = m.combo + combo_off(m.C, i, p.mask);
      gx = rec[0];
      gy = rec[1];
      for (int k = 0; k < 3; ++k) off[k] = rec[5 + k];
    }
  } else {
    J = aw.pwjac + i;
    w0 = J->w0;
    if (J->plane) {
      const Pw2Rec& r = m.pw2[i];
      gx = J->gx;
      gy = J->gy;
      for (int k = 0; k < 3; ++k) off[k] = gx * r.dedge[k][0] + gy * r.dedge[k][1];
    }
  }
  // slot reverses
  double lw0 = 0., lgx = 0., lgy = 0., loff[3];
  for (int k = 0; k < 3; ++k) {
    const int slot = k * C + i;
    double law, lu0, lv0, lgxk, lgyk, lze;
    slot_reverse<COR0>(m.ze[slot], w0 + off[k], u, v, cor, aw.lew[slot], aw.leu[slot], aw.lev[slot], aw.lsx[slot],
                 aw.lsy[slot], &law, &lu0, &lv0, &lgxk, &lgyk, &lze);
    lw0 += law;
    loff[k] = law;
    lu_i += lu0;
    lv_i += lv0;
    lgx += lgxk;
    lgy += lgyk;
    lam_edge_z(m, aw, i, k, lze + aw.lze[slot]);
  }
  if (p.type == 2) {
    lw_i += lw0;
    if (p.kept) {
      // the combination plane through neighbour centroids / edge centres:
      // off_k = g0 dEx + g1 dEy
      const Pw2Rec& r = m.pw2[i];
      double lg0 = lgx, lg1 = lgy;
      for (int k = 0; k < 3; ++k) {
        lg0 = fma(loff[k], r.dedge[k][0], lg0);
        lg1 = fma(loff[k], r.dedge[k][1], lg1);
      }
      const double* T = aw.padj + (size_t)i * 48 + p.mask * 6;
      const double lp[3] = {fma(lg0, T[0], lg1 * T[3]), fma(lg0, T[1], lg1 * T[4]), fma(lg0, T[2], lg1 * T[5])};
      combo_points_to_nodes(m, aw, i, p.mask, lp);
    }
  } else if (!J->plane) {
    // PartWet1 level over (w, z0, z1, z2)
    lw_i = fma(lw0, J->jw0[0], lw_i);
    for (int q = 0; q < 3; ++q)
      if (J->jw0[1 + q] != 0.) atomicAdd(aw.lz + cnode(m, i, q), lw0 * J->jw0[1 + q]);
  } else {
    const Pw2Rec& r = m.pw2[i];
    double lg0 = lgx, lg1 = lgy;
    for (int k = 0; k < 3; ++k) {
      lg0 = fma(loff[k], r.dedge[k][0], lg0);
      lg1 = fma(loff[k], r.dedge[k][1], lg1);
    }
    double g[5];
    for (int q = 0; q < 5; ++q) g[q] = fma(lw0, J->jw0[q], fma(lg0, J->jgx[q], lg1 * J->jgy[q]));
    lw_i += g[0];
    // node z of the sorted vertices
    for (int s = 0; s < 3; ++s)
      if (g[2 + s] != 0.) atomicAdd(aw.lz + cnode(m, i, r.sk[s]), g[2 + s]);
    // w23 through the cell that supplied the node maximum
    const double g1 = g[1];
    if (g1 != 0.) {
      const int t = J->target;
      switch (J->route) {
        case 0: atomicAdd(aw.lz + gidx(m, t, m.N), g1); break;
        case 1:
          for (int q = 0; q < 3; ++q) atomicAdd(aw.lz + cnode(m, gidx(m, t, C), q), g1 * J->rc[q]);
          break;
        case 2:
          atomicAdd(aw.lscatter + gidx(m, t, C), g1);
          if (J->mask >= 0) {
            const double lp[3] = {g1 * J->rc[0], g1 * J->rc[1], g1 * J->rc[2]};
            combo_points_to_nodes(m, aw, gidx(m, t, C), J->mask, lp);
          }
          break;
        default:
          atomicAdd(aw.lscatter + gidx(m, t, C), g1 * J->rc[0]);
          for (int q = 0; q < 3; ++q)
            if (J->rc[1 + q] != 0.) atomicAdd(aw.lz + cnode(m, gidx(m, t, C), q), g1 * J->rc[1 + q]);
          break;
      }
    }
  }
  aw.lamp[i] += lw_i;
  aw.lamp[C + i] += lu_i;
  aw.lamp[2 * C + i] += lv_i;
  lam_cell_z(m, aw, i, lbc);
}

template <bool COR0>
__global__ void __launch_bounds__(256, 4) k_adj_recon(DevMesh m, DevWork wk, AdjWork aw, const double* W,
                                                   const double* U, const double* V, int batched) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m.C) adj_recon_cell<COR0>(m, wk, aw, W, U, V, i, batched);
}

// Jacobians of the stage's partially-wet cells (the list pass 1 of the forward
// wrote), one warp per block so that the few listed cells spread over the SMs
__global__ void __launch_bounds__(32) k_pw_jacobian(DevMesh m, DevWork wk, AdjWork aw, const double* W) {
  const int n = min(*wk.pwcount, m.C);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int i = gidx(m, wk.pwlist[q], m.C);
    pw_jacobian(m, wk, aw, W, i, aw.pwjac + i);
  }
}

}  // namespace

// ----------------------------------------------------------------- driver
struct AdjointState {
  AdjWork aw{};
  std::vector<void*> allocs;
  // tape of the last taped forward run
  int scheme = 1;
  Scheme sc{};  // the scheme's table at the taped run
  int64_t n_steps = 0, ckpt = 0, obs = 0;
  int n_gauges = 0;
  int* d_gauges = nullptr;
  std::vector<double*> checkpoints;  // [3C] state at steps 0, ckpt, 2 ckpt, ...
  double* d_dt = nullptr;            // [n_steps] recorded dt
  double* d_traces = nullptr;        // [n_obs x n_gauges]
  bool taped = false;
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  template <class T>
  T* alloc(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (T*)p;
  }
  void free_tape() {
    for (double* p : checkpoints) cudaFree(p);
    checkpoints.clear();
    if (d_dt) cudaFree(d_dt);
    if (d_traces) cudaFree(d_traces);
    if (d_gauges) cudaFree(d_gauges);
    d_dt = d_traces = nullptr;
    d_gauges = nullptr;
    taped = false;
  }
  ~AdjointState() {
    free_tape();
    for (void* p : allocs) cudaFree(p);
    if (side) cudaStreamDestroy(side);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
  }
};

void adjoint_state_delete(AdjointState* a) { delete a; }

std::string Engine::adjoint_init() {
  if (adj_) return "";
  AdjointState* a = new AdjointState();
  const int64_t C = mesh_.C, E = mesh_.E, N = mesh_.N;
  AdjWork& w = a->aw;
  bool ok = true;
  auto A = [&](double*& p, size_t n) {
    p = a->alloc<double>(n);
    ok = ok && p;
  };
  A(w.lam, 3 * C); A(w.lamp, 3 * C); A(w.lam0, 3 * C);
  A(w.lew, 3 * C); A(w.leu, 3 * C); A(w.lev, 3 * C); A(w.lsx, 3 * C); A(w.lsy, 3 * C); A(w.lze, 3 * C);
  A(w.lF0, 3 * C); A(w.lF1, 3 * C); A(w.lF2, 3 * C); A(w.lF0d, 3 * C); A(w.ldtk, 3 * C); A(w.lhwall, 3 * C);
  A(w.lbc, C); A(w.lscatter, C); A(w.lz, N);
  w.pwjac = a->alloc<PwJac>(C);
  w.padj = a->alloc<double>(48 * C);
  ok = ok && w.pwjac && w.padj;
  w.route = a->alloc<unsigned char>(3 * C);
  ok = ok && w.route;
  // twin slots, node -> cells, edge nodes over all instances (global ids:
  // each instance's local index plus its offset)
  std::vector<int> twin(3 * C, -1), eown_k(E, -1), enb_k(E, -1), en(2 * E);
  std::vector<int> ptr(N + 1, 0), cells(3 * C);
  for (int q = 0; q < I(); ++q) {
    const HostInstance& h = host[q];
    const int64_t c0 = cell_off[q], e0 = edge_off[q], n0 = node_off[q];
    for (int64_t e = 0; e < h.E; ++e) {
      en[2 * (e0 + e)] = (int)(n0 + h.en[2 * e]);
      en[2 * (e0 + e) + 1] = (int)(n0 + h.en[2 * e + 1]);
    }
    for (int64_t i = 0; i < h.C; ++i)
      for (int k = 0; k < 3; ++k) {
        const int64_t e = h.ce[3 * i + k];
        if (h.ec[2 * e] == i) eown_k[e0 + e] = (int)(k * C + c0 + i);
        else enb_k[e0 + e] = (int)(k * C + c0 + i);
        ptr[n0 + h.cn[3 * i + k] + 1]++;
      }
  }
  for (int64_t e = 0; e < E; ++e)
    if (eown_k[e] >= 0 && enb_k[e] >= 0) {
      twin[eown_k[e]] = enb_k[e];
      twin[enb_k[e]] = eown_k[e];
    }
  for (int64_t n = 0; n < N; ++n) ptr[n + 1] += ptr[n];
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int q = 0; q < I(); ++q) {
    const HostInstance& h = host[q];
    const int64_t c0 = cell_off[q], n0 = node_off[q];
    for (int64_t i = 0; i < h.C; ++i)
      for (int k = 0; k < 3; ++k) cells[fill[n0 + h.cn[3 * i + k]]++] = (int)(((c0 + i) << 2) | k);
  }
  // Each node's cells in the caller's cell order: where several cells attain
  // the node maximum, the reverse routes through the first of them, and that
  // choice must not depend on the device order the tuner picked.
  {
    std::vector<int64_t> caller((size_t)C);
    for (int q = 0; q < I(); ++q) {
      const Layout* L = (size_t)q < layouts.size() ? &layouts[q] : nullptr;
      const bool id = !L || L->identity();
      for (int64_t j = 0; j < cell_off[q + 1] - cell_off[q]; ++j)
        caller[cell_off[q] + j] = cell_off[q] + (id ? j : L->cell_from[j]);
    }
    for (int64_t n = 0; n < N; ++n)
      std::sort(cells.begin() + ptr[n], cells.begin() + ptr[n + 1],
                [&](int a, int b) { return caller[a >> 2] < caller[b >> 2]; });
  }
  int* d_twin = a->alloc<int>(3 * C);
  int* d_ptr = a->alloc<int>(N + 1);
  int* d_cells = a->alloc<int>(3 * C);
  int* d_en = a->alloc<int>(2 * E);
  ok = ok && d_twin && d_ptr && d_cells && d_en;
  if (!ok) {
    delete a;
    return "adjoint work allocation failed";
  }
  cudaMemcpy(d_twin, twin.data(), 3 * C * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(d_ptr, ptr.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(d_cells, cells.data(), 3 * C * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(d_en, en.data(), 2 * E * sizeof(int), cudaMemcpyHostToDevice);
  w.twin = d_twin;
  w.node_ptr = d_ptr;
  w.node_cells = d_cells;
  w.edge_nodes = d_en;
  cudaMemset(w.lscatter, 0, C * sizeof(double));
  k_plane_adj_init<<<(int)((C + 255) / 256), 256, 0, stream_>>>(mesh_, w.padj);
  if (cudaStreamSynchronize(stream_) != cudaSuccess) {
    delete a;
    return "adjoint table set-up failed";
  }
  if (cudaStreamCreateWithFlags(&a->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&a->ev_join, cudaEventDisableTiming) != cudaSuccess) {
    delete a;
    return "adjoint stream set-up failed";
  }
  adj_ = a;
  return "";
}

std::string Engine::adjoint_forward(int scheme, int64_t n_steps, int64_t ckpt, const int* gauges, int n_gauges,
                                    int64_t obs, double* traces_host, bool traces_device) {
  std::string err = adjoint_init();
  if (!err.empty()) return err;
  AdjointState& a = *adj_;
  a.free_tape();
  const int64_t C = mesh_.C;
  a.scheme = scheme;
  a.sc = scheme_of(scheme);
  a.n_steps = n_steps;
  a.ckpt = ckpt;
  a.obs = obs;
  a.n_gauges = n_gauges;
  const int64_t n_obs = obs > 0 ? n_steps / obs : 0;
  const int64_t NI = I();
  if (cudaMalloc(&a.d_dt, (n_steps ? n_steps : 1) * NI * sizeof(double)) != cudaSuccess) return "tape allocation failed";
  if (cudaMalloc(&a.d_traces, (n_obs * n_gauges ? n_obs * n_gauges : 1) * sizeof(double)) != cudaSuccess)
    return "tape allocation failed";
  if (cudaMalloc(&a.d_gauges, (n_gauges ? n_gauges : 1) * sizeof(int)) != cudaSuccess) return "tape allocation failed";
  cudaMemcpy(a.d_gauges, gauges, n_gauges * sizeof(int), cudaMemcpyHostToDevice);
  // every checkpoint allocated up front (no allocation inside the run)
  const int64_t n_ckpt = n_steps > 0 ? (n_steps + ckpt - 1) / ckpt : 0;
  for (int64_t q = 0; q < n_ckpt; ++q) {
    double* cp = nullptr;
    if (cudaMalloc(&cp, 3 * C * sizeof(double)) != cudaSuccess) return "checkpoint allocation failed";
    a.checkpoints.push_back(cp);
  }
  for (int64_t n = 0; n < n_steps; ++n) {
    if (n % ckpt == 0) {
      double* cp = a.checkpoints[n / ckpt];
      for (int q = 0; q < 3; ++q)
        cudaMemcpyAsync(cp + q * C, state(0, q), C * sizeof(double), cudaMemcpyDeviceToDevice, stream_);
    }
    // the plain step's CUDA graph (dt = CFLdt() of the previous flux pass)
    cudaError_t e = run_graph(scheme, 1, 1);
    if (e != cudaSuccess) return std::string("forward step: ") + cudaGetErrorString(e);
    cudaMemcpyAsync(a.d_dt + n * NI, work_.dt, NI * sizeof(double), cudaMemcpyDeviceToDevice, stream_);
    if (obs > 0 && (n + 1) % obs == 0 && n_gauges > 0) {
      const int64_t j = (n + 1) / obs - 1;
      k_gather_gauges<<<(n_gauges + 255) / 256, 256, 0, stream_>>>(state(0, 0), a.d_gauges, n_gauges,
                                                                    a.d_traces + j * n_gauges);
      ++launches_;
    }
  }
  if (traces_host && n_obs * n_gauges > 0)
    cudaMemcpyAsync(traces_host, a.d_traces, n_obs * n_gauges * sizeof(double),
                    traces_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream_);
  cudaError_t e = cudaStreamSynchronize(stream_);
  if (e != cudaSuccess) return std::string("taped forward run: ") + cudaGetErrorString(e);
  a.taped = true;
  return "";
}

std::string Engine::run_traces(int scheme, int64_t n_steps, const double* dts_host, const int* gauges, int n_gauges,
                               int64_t obs, double* traces_host) {
  const int64_t NI = I();
  const int64_t n_obs = obs > 0 ? n_steps / obs : 0;
  double *d_dts = nullptr, *d_tr = nullptr;
  int* d_g = nullptr;
  std::string err;
  auto release = [&] {
    if (d_dts) cudaFree(d_dts);
    if (d_tr) cudaFree(d_tr);
    if (d_g) cudaFree(d_g);
  };
  if (cudaMalloc(&d_dts, (n_steps ? n_steps : 1) * NI * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_tr, (n_obs * n_gauges ? n_obs * n_gauges : 1) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_g, (n_gauges ? n_gauges : 1) * sizeof(int)) != cudaSuccess) {
    release();
    return "allocation failed";
  }
  cudaError_t e = cudaMemcpyAsync(d_dts, dts_host, n_steps * NI * sizeof(double), cudaMemcpyHostToDevice, stream_);
  if (e == cudaSuccess && n_gauges)
    e = cudaMemcpyAsync(d_g, gauges, n_gauges * sizeof(int), cudaMemcpyHostToDevice, stream_);
  for (int64_t n = 0; n < n_steps && e == cudaSuccess; ++n) {
    // the step's dt per instance, then one replay of the fixed-dt step graph
    e = cudaMemcpyAsync(d_fixed_dt, d_dts + n * NI, NI * sizeof(double), cudaMemcpyDeviceToDevice, stream_);
    if (e == cudaSuccess) e = run_graph(scheme, 2, 1);
    if (e == cudaSuccess && obs > 0 && (n + 1) % obs == 0 && n_gauges > 0) {
      const int64_t j = (n + 1) / obs - 1;
      k_gather_gauges<<<(n_gauges + 255) / 256, 256, 0, stream_>>>(state(0, 0), d_g, n_gauges, d_tr + j * n_gauges);
      ++launches_;
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess && traces_host && n_obs * n_gauges > 0)
    e = cudaMemcpyAsync(traces_host, d_tr, n_obs * n_gauges * sizeof(double), cudaMemcpyDeviceToHost, stream_);
  cudaError_t e2 = cudaStreamSynchronize(stream_);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) err = std::string("trace run: ") + cudaGetErrorString(e);
  release();
  return err;
}

std::string Engine::caller_maps() {
  if (d_cell_caller && d_node_caller) return "";
  std::vector<int> cm((size_t)mesh_.C), nm((size_t)mesh_.N);
  for (size_t q = 0; q < host.size(); ++q) {
    const Layout* L = q < layouts.size() ? &layouts[q] : nullptr;
    const bool id = !L || L->identity();
    for (int64_t j = 0; j < cell_off[q + 1] - cell_off[q]; ++j)
      cm[cell_off[q] + j] = (int)(cell_off[q] + (id ? j : L->cell_from[j]));
    for (int64_t j = 0; j < node_off[q + 1] - node_off[q]; ++j)
      nm[node_off[q] + j] = (int)(node_off[q] + (id ? j : L->node_from[j]));
  }
  d_cell_caller = dalloc<int>(cm.size());
  d_node_caller = dalloc<int>(nm.size());
  if (!d_cell_caller || !d_node_caller) return "device allocation failed";
  if (cudaMemcpy(d_cell_caller, cm.data(), cm.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_node_caller, nm.data(), nm.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return std::string("uploading the caller order: ") + cudaGetErrorString(cudaGetLastError());
  return "";
}

std::string Engine::adjoint_dts(double* out_host) {
  if (!adj_ || !adj_->taped) return "no taped forward run";
  cudaError_t e = cudaMemcpy(out_host, adj_->d_dt, adj_->n_steps * I() * sizeof(double), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? "" : cudaGetErrorString(e);
}

__global__ void k_interleave(const double* W, int C, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < C) {
    out[3 * i] = W[i];
    out[3 * i + 1] = W[C + i];
    out[3 * i + 2] = W[2 * C + i];
  }
}

// out[w * map[i] + c] = in[w * i + c]: device rows to the caller's order
__global__ void k_rows_to_caller(const double* in, const int* map, int n, int w, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    for (int c = 0; c < w; ++c) out[(size_t)w * map[i] + c] = in[(size_t)w * i + c];
}

std::string Engine::adjoint_backward(const double* trace_grads_host, double* grad_prim_host, double* grad_z_host,
                                     bool device) {
  if (!adj_ || !adj_->taped) return "no taped forward run to differentiate";
  if (device) {
    std::string e = caller_maps();
    if (!e.empty()) return e;
  }
  AdjointState& a = *adj_;
  AdjWork& w = a.aw;
  w.reg_depth = adj_reg_depth_;
  const int64_t C = mesh_.C, N = mesh_.N;
  const Scheme sc = a.sc;
  const int ns = sc.n;
  const int64_t n_obs = a.obs > 0 ? a.n_steps / a.obs : 0;
  double* d_tg = nullptr;
  if (cudaMalloc(&d_tg, (n_obs * a.n_gauges ? n_obs * a.n_gauges : 1) * sizeof(double)) != cudaSuccess)
    return "allocation failed";
  if (n_obs * a.n_gauges)
    cudaMemcpy(d_tg, trace_grads_host, n_obs * a.n_gauges * sizeof(double),
               device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice);
  // stage-input store of one segment: [K][ns] states of 3C, plus the segment end
  const int64_t K = a.ckpt;
  std::vector<double*> store((size_t)K * ns + 1, nullptr);
  for (auto& p : store)
    if (cudaMalloc(&p, 3 * C * sizeof(double)) != cudaSuccess) {
      cudaFree(d_tg);
      for (auto& q : store)
        if (q) cudaFree(q);
      return "segment store allocation failed";
    }
  const int b = 256, gc = (int)((C + b - 1) / b);
  // per-stage forward intermediates of one segment (interface slots, fluxes,
  // draining dt, node maxima, part-wet list) when device memory allows
  const int64_t E = mesh_.E;
  const size_t per_stage = ((15 * C + 10 * E + 5 * C) * sizeof(double) + N * sizeof(unsigned long long) +
                            (C + 1) * sizeof(int) + C + 255) / 256 * 256;
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const bool keep = (double)per_stage * (double)(K * ns) < 0.6 * (double)free_b;
  std::vector<DevWork> kept;
  std::vector<double*> kept_n;  // state before ConsAssigner of each stage
  char* kept_pool = nullptr;
  if (keep) {
    if (cudaMalloc(&kept_pool, per_stage * (size_t)(K * ns)) != cudaSuccess) {
      cudaFree(d_tg);
      for (auto& q : store) cudaFree(q);
      return "intermediate store allocation failed";
    }
    kept.resize((size_t)(K * ns));
    kept_n.resize((size_t)(K * ns));
    for (int64_t q = 0; q < K * ns; ++q) {
      char* p = kept_pool + per_stage * (size_t)q;
      DevWork wq = work_;
      auto take = [&](size_t bytes) {
        char* r = p;
        p += bytes;
        return r;
      };
      wq.ew = (double*)take(3 * C * sizeof(double));
      wq.eu = (double*)take(3 * C * sizeof(double));
      wq.ev = (double*)take(3 * C * sizeof(double));
      wq.sx = (double*)take(3 * C * sizeof(double));
      wq.sy = (double*)take(3 * C * sizeof(double));
      wq.f0 = (double*)take(E * sizeof(double));
      wq.f1 = (double*)take(E * sizeof(double));
      wq.f2 = (double*)take(E * sizeof(double));
      wq.ftape = (double*)take(7 * E * sizeof(double));
      wq.drain = (double*)take(C * sizeof(double));
      wq.pwrec = (double*)take(C * sizeof(double));
      wq.maxwp = (unsigned long long*)take(N * sizeof(unsigned long long));
      wq.pwlist = (int*)take(C * sizeof(int));
      kept_n[q] = (double*)take(3 * C * sizeof(double));
      wq.pwcount = (int*)take(sizeof(int));
      wq.cls = (unsigned char*)take((size_t)C);
      kept[q] = wq;
    }
  }
  cudaMemsetAsync(w.lam, 0, 3 * C * sizeof(double), stream_);
  cudaMemsetAsync(w.lz, 0, N * sizeof(double), stream_);
  cudaMemsetAsync(w.lscatter, 0, C * sizeof(double), stream_);
  std::vector<double> tsum_saved((size_t)I(), 0.);  // the recompute must not advance the clocks
  cudaMemcpyAsync(tsum_saved.data(), work_.tsum, I() * sizeof(double), cudaMemcpyDeviceToHost, stream_);
  cudaStreamSynchronize(stream_);
  double* lam_step = nullptr;  // adjoint of the current step's end state
  cudaMalloc(&lam_step, 3 * C * sizeof(double));
  cudaMemsetAsync(lam_step, 0, 3 * C * sizeof(double), stream_);
  std::string err;
  const int64_t nseg = (a.n_steps + K - 1) / K;
  // The first step index of the current segment lives on the device, so that
  // one captured graph of a full segment's recompute and one of its reverse
  // replay for every full segment.
  long long* d_s0 = nullptr;
  if (cudaMalloc(&d_s0, sizeof(long long)) != cudaSuccess) err = "allocation failed";
  const bool seeds = a.obs > 0 && a.n_gauges > 0;
  // recompute of steps s0 .. s0+len-1 with the recorded dt, keeping every
  // stage's forward intermediates when they fit
  auto enqueue_recompute = [&](int64_t len) -> cudaError_t {
    for (int64_t loc = 0; loc < len; ++loc) {
      const int64_t base = loc * ns;
      k_fetch_dt<<<(I() + 127) / 128, 128, 0, stream_>>>(d_fixed_dt, a.d_dt, d_s0, loc, I());
      double* S0p = store[base];
      const double* u0[3] = {S0p, S0p + C, S0p + 2 * C};
      for (int s = 0; s < ns; ++s) {
        double* inp = store[base + s];
        double* outp = store[base + s + 1];
        const double* in[3] = {inp, inp + C, inp + 2 * C};
        double* out[3] = {outp, outp + C, outp + 2 * C};
        cudaError_t e;
        if (keep) {
          const DevWork saved = work_;
          work_ = kept[base + s];
          e = reset_pass();
          if (e == cudaSuccess) {
            // the plain stage's kernels with PartWet2 and the fluxes next to
            // partially-wet cells on the side stream, keeping every
            // intermediate (k_drain_keep leaves the node maxima and the list)
            launch_recon1(in[0], in[1], in[2], s == 0 ? 2 : 0);
            cudaEventRecord(ev_fork_, stream_);
            cudaStreamWaitEvent(side_, ev_fork_, 0);
            launch_recon2(in[0], in[1], in[2], side_);
            fluxes_pw(in[0], side_);
            cudaEventRecord(ev_join_, side_);
            e = fluxes(in[0], 1);
            cudaStreamWaitEvent(stream_, ev_join_, 0);
          }
          if (e == cudaSuccess) {
            k_drain_keep<<<gc, b, 0, stream_>>>(mesh_, work_, in[0]);
            e = update_only(sc.s[s], in, u0, out, kept_n[base + s]);
          }
          work_ = saved;
        } else {
          e = reset_pass();
          if (e == cudaSuccess) e = launch_stage(sc.s[s], in, u0, out, s == 0, s == 0 ? 2 : 0);
        }
        if (e != cudaSuccess) return e;
      }
    }
    return cudaGetLastError();
  };
  // reverse of steps s0+len-1 .. s0
  auto enqueue_reverse = [&](int64_t len) -> cudaError_t {
    for (int64_t loc = len - 1; loc >= 0; --loc) {
      const int64_t base = loc * ns;
      if (seeds)
        k_seed_gauges_seg<<<(a.n_gauges + 255) / 256, 256, 0, stream_>>>(lam_step, a.d_gauges, a.n_gauges, d_tg,
                                                                         d_s0, loc, a.obs);
      k_fetch_dt<<<(I() + 127) / 128, 128, 0, stream_>>>(work_.dt, a.d_dt, d_s0, loc, I());
      double* S0p = store[base];
      const double* u0[3] = {S0p, S0p + C, S0p + 2 * C};
      cudaMemsetAsync(w.lam0, 0, 3 * C * sizeof(double), stream_);
      cudaMemcpyAsync(w.lam, lam_step, 3 * C * sizeof(double), cudaMemcpyDeviceToDevice, stream_);
      for (int s = ns - 1; s >= 0; --s) {
        double* inp = store[base + s];
        const double* in[3] = {inp, inp + C, inp + 2 * C};
        cudaMemsetAsync(w.lamp, 0, 3 * C * sizeof(double), stream_);
        cudaError_t e = keep ? adjoint_stage_reverse_stored(sc.s[s], in, u0, w, kept[base + s], kept_n[base + s])
                             : adjoint_stage_reverse(sc.s[s], in, u0, w);
        if (e != cudaSuccess) return e;
        k_fold_scatter<<<gc, b, 0, stream_>>>((int)C, w.lamp, w.lscatter);
        cudaMemcpyAsync(w.lam, w.lamp, 3 * C * sizeof(double), cudaMemcpyDeviceToDevice, stream_);
      }
      // adjoint of the step's initial state: through the first stage's input and the Shu-Osher terms
      k_add3<<<gc, b, 0, stream_>>>((int)C, w.lam, w.lam0, lam_step);
    }
    return cudaGetLastError();
  };
  // captures body() on a private stream; null graph if capture fails
  auto capture = [&](auto&& body) -> cudaGraphExec_t {
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    const cudaStream_t saved = stream_;
    stream_ = cap;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    if (cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const cudaError_t e = body();
      const cudaError_t e2 = cudaStreamEndCapture(cap, &g);
      if (e == cudaSuccess && e2 == cudaSuccess && cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) ge = nullptr;
      if (g) cudaGraphDestroy(g);
    }
    stream_ = saved;
    cudaStreamDestroy(cap);
    cudaGetLastError();
    return ge;
  };
  cudaGraphExec_t g_rec = nullptr, g_rev = nullptr;
  bool tried = false;
  for (int64_t seg = nseg - 1; seg >= 0 && err.empty(); --seg) {
    const int64_t s0 = seg * K, s1 = std::min(a.n_steps, s0 + K), len = s1 - s0;
    for (int q = 0; q < 3; ++q)
      cudaMemcpyAsync(store[0] + q * C, a.checkpoints[seg] + q * C, C * sizeof(double), cudaMemcpyDeviceToDevice,
                      stream_);
    k_set_i64<<<1, 32, 0, stream_>>>(d_s0, s0);
    if (len == K && !tried) {
      tried = true;
      g_rec = capture([&] { return enqueue_recompute(K); });
      g_rev = capture([&] { return enqueue_reverse(K); });
    }
    cudaError_t e = (len == K && g_rec) ? cudaGraphLaunch(g_rec, stream_) : enqueue_recompute(len);
    if (e != cudaSuccess) {
      err = std::string("segment recompute: ") + cudaGetErrorString(e);
      break;
    }
    e = (len == K && g_rev) ? cudaGraphLaunch(g_rev, stream_) : enqueue_reverse(len);
    if (e != cudaSuccess) err = std::string("stage reverse: ") + cudaGetErrorString(e);
  }
  if (g_rec) cudaGraphExecDestroy(g_rec);
  if (g_rev) cudaGraphExecDestroy(g_rev);
  if (err.empty()) {
    double* d_out = store[0];
    k_interleave<<<gc, b, 0, stream_>>>(lam_step, (int)C, d_out);
    if (device) {
      k_rows_to_caller<<<gc, b, 0, stream_>>>(d_out, d_cell_caller, (int)C, 3, grad_prim_host);
      k_rows_to_caller<<<(int)((N + b - 1) / b), b, 0, stream_>>>(w.lz, d_node_caller, (int)N, 1, grad_z_host);
      launches_ += 2;
    } else {
      cudaMemcpyAsync(grad_prim_host, d_out, 3 * C * sizeof(double), cudaMemcpyDeviceToHost, stream_);
      cudaMemcpyAsync(grad_z_host, w.lz, N * sizeof(double), cudaMemcpyDeviceToHost, stream_);
    }
    cudaError_t e = cudaStreamSynchronize(stream_);
    if (e != cudaSuccess) err = std::string("adjoint: ") + cudaGetErrorString(e);
  }
  cudaMemcpy(work_.tsum, tsum_saved.data(), I() * sizeof(double), cudaMemcpyHostToDevice);
  if (kept_pool) cudaFree(kept_pool);
  for (auto& p : store) cudaFree(p);
  cudaFree(d_tg);
  cudaFree(lam_step);
  cudaFree(d_s0);
  return err;
}

// Threads per block of the reverse kernels: 128 (and 64) measured 3 % faster
// backward passes than 256 on a 250k-cell mesh (1.83 vs 1.89 s for 2000 steps).
// k_adj_update, k_adj_flux and k_adj_recon are held at 64 registers
// (__launch_bounds__(256, 4); 80-97 uncapped): on the 64-instance, 3.85M-cell
// batch over 500 steps the backward took 5.43 s against 5.49-5.51 s uncapped
// and 5.43-5.46 s at 72 or 80, with the same gradients.
constexpr int kReverseBlock = 128;

cudaError_t Engine::adjoint_stage_reverse(const Stage& st, const double* const* in, const double* const* u0,
                                          AdjWork& aw) {
  // recompute the stage's forward intermediates from its input into work_
  cudaError_t e = reset_pass();
  if (e == cudaSuccess) e = interface_values(in[0], in[1], in[2], 0);
  if (e == cudaSuccess) e = fluxes(in[0]);
  if (e != cudaSuccess) return e;
  const int b = kReverseBlock;
  k_drain_keep<<<(mesh_.C + b - 1) / b, b, 0, stream_>>>(mesh_, work_, in[0]);
  ++launches_;
  return adjoint_stage_reverse_stored(st, in, u0, aw, work_, nullptr);
}

cudaError_t Engine::adjoint_stage_reverse_stored(const Stage& st, const double* const* in, const double* const* u0,
                                                 AdjWork& aw, const DevWork& wk, const double* nst) {
  const int b = kReverseBlock;
  const int gc = (mesh_.C + b - 1) / b, ge = (mesh_.E + b - 1) / b;
  // the partially-wet cells' Jacobians need no adjoint: a side stream
  // computes them while R1-R3 run
  AdjointState& a = *adj_;
  cudaEventRecord(a.ev_fork, stream_);
  cudaStreamWaitEvent(a.side, a.ev_fork, 0);
  const int gpw = std::max(1, std::min((mesh_.C + 31) / 32, 152 * 16));
  k_pw_jacobian<<<gpw, 32, 0, a.side>>>(mesh_, wk, aw, in[0]);
  cudaEventRecord(a.ev_join, a.side);
  k_adj_update<<<gc, b, 0, stream_>>>(mesh_, wk, aw, in[0], in[1], in[2], u0[0], u0[1], u0[2], nst, st, batched_);
  k_adj_drain<<<gc, b, 0, stream_>>>(mesh_, wk, aw, in[0]);
  switch (flux_ * 3 + ws_) {
    case 0: k_adj_flux<0, 0><<<ge, b, 0, stream_>>>(mesh_, wk, aw, in[0]); break;
    case 1: k_adj_flux<0, 1><<<ge, b, 0, stream_>>>(mesh_, wk, aw, in[0]); break;
    case 2: k_adj_flux<0, 2><<<ge, b, 0, stream_>>>(mesh_, wk, aw, in[0]); break;
    case 3: k_adj_flux<1, 0><<<ge, b, 0, stream_>>>(mesh_, wk, aw, in[0]); break;
    case 4: k_adj_flux<1, 1><<<ge, b, 0, stream_>>>(mesh_, wk, aw, in[0]); break;
    default: k_adj_flux<1, 2><<<ge, b, 0, stream_>>>(mesh_, wk, aw, in[0]); break;
  }
  cudaStreamWaitEvent(stream_, a.ev_join, 0);
  if (cor0_) k_adj_recon<true><<<gc, b, 0, stream_>>>(mesh_, wk, aw, in[0], in[1], in[2], batched_);
  else k_adj_recon<false><<<gc, b, 0, stream_>>>(mesh_, wk, aw, in[0], in[1], in[2], batched_);
  launches_ += 5;
  return cudaGetLastError();
}

}  // namespace swe
