// swe_precompute.cu -- host-side validation and static geometry of one mesh.
//
// Everything the reference recomputes on each call from node positions alone
// (Domain::T / E / Norm / Tang / L / Area / TriangSlope, src/Bathymetry.cpp:
// 10-90, and the parts of MUSCLObject's reconstructions that depend on the
// mesh only, src/MUSCLObject.cpp:31-191) is evaluated here once, with the
// reference's operation order and without FMA contraction (-ffp-contract=off
// on the host compiler), so the device kernels see the same bits the CPU
// restatement computes on the fly.
#include <algorithm>
#include <cmath>
#include <limits>
#include <string>
#include <thread>
#include <vector>

#include "swe_engine.cuh"

namespace swe {

void HostImage::resize(int C_, int E_, int N_, int I_) {
  C = C_; E = E_; N = N_; I = I_;
  cnode.assign(3 * (size_t)C, 0); cnbr.assign(3 * (size_t)C, -1); cedge.assign(3 * (size_t)C, 0);
  cinst.assign(C, 0); cown.assign(C, 0);
  bc.assign(C, 0); fwthr.assign(C, 0); area.assign(C, 0);
  zn.assign(3 * (size_t)C, 0); ze.assign(3 * (size_t)C, 0); cek.assign(3 * (size_t)C, 0);
  cnxc.assign(3 * (size_t)C, 0); cnyc.assign(3 * (size_t)C, 0);
  dry.assign((size_t)C * kDryStride, 0); combo.assign((size_t)C * 8 * kComboStride, 0);
  pw1.assign((size_t)C * kPw1Stride, 0); pw2.assign(C, Pw2Rec{});
  srec.assign(3 * (size_t)C, SlotRec{}); cslot.assign(3 * (size_t)C, int2{0, -1});
  erec.assign(E, EdgeRec{}); eidx.assign(E, int4{0, -1, 0, -1});
  eown.assign(E, 0); enb.assign(E, -1); eslotl.assign(E, 0); eslotr.assign(E, -1); einst.assign(E, 0);
  enx.assign(E, 0); eny.assign(E, 0); etx.assign(E, 0); ety.assign(E, 0); ezm.assign(E, 0); elmin.assign(E, 0);
  nz.assign(N, 0);
  nptr.assign((size_t)N + 1, 0); ncell.assign(3 * (size_t)C, 0);
  inst_cell_begin.assign(I, 0); inst_cfl.assign(I, 0); inst_cor.assign(I, 0);
}

namespace {

struct Geo {
  const HostInstance& h;
  const double* P(int64_t n) const { return h.geom.data() + 3 * n; }
  // src/Bathymetry.cpp:24-27
  void T(int64_t t, double out[3]) const {
    const int64_t* tp = h.cn.data() + 3 * t;
    const double k = 1. / 3.;
    for (int r = 0; r < 3; ++r) out[r] = P(tp[0])[r] * k + P(tp[1])[r] * k + P(tp[2])[r] * k;
  }
  // edge centre = midpoint of the edge's nodes (Domain::E is a stub in the reference)
  void Emid(int64_t e, double out[3]) const {
    const double* a = P(h.en[2 * e]);
    const double* b = P(h.en[2 * e + 1]);
    for (int r = 0; r < 3; ++r) out[r] = (a[r] + b[r]) * 0.5;
  }
  // src/Bathymetry.cpp:82-85, src/PointOperations.cpp:4-6
  double L(int64_t e) const {
    const double* a = P(h.en[2 * e]);
    const double* b = P(h.en[2 * e + 1]);
    return sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]));
  }
  // src/Bathymetry.cpp:87-90, src/PointOperations.cpp:8-14
  double Area(int64_t t) const {
    const int64_t* tp = h.cn.data() + 3 * t;
    const double *a = P(tp[0]), *b = P(tp[1]), *c = P(tp[2]);
    double ba0 = b[0] - a[0], ba1 = b[1] - a[1];
    double ca0 = c[0] - a[0], ca1 = c[1] - a[1];
    return 0.5 * fabs(ba0 * ca1 - ca0 * ba1);
  }
  // src/Bathymetry.cpp:69-76
  void Tang(int64_t e, int64_t t, double out[2]) const {
    const double* p0 = P(h.en[2 * e]);
    const double* p1 = P(h.en[2 * e + 1]);
    double l = L(e);
    double tan0 = (p1[0] - p0[0]) / l, tan1 = (p1[1] - p0[1]) / l;
    double tt[3];
    T(t, tt);
    double d0 = tt[0] - p0[0], d1 = tt[1] - p0[1];
    if (d0 * tan1 - tan0 * d1 > 0.) {
      tan0 = -tan0;
      tan1 = -tan1;
    }
    out[0] = tan0;
    out[1] = tan1;
  }
  // src/Bathymetry.cpp:78-80
  void Norm(int64_t e, int64_t t, double out[2]) const {
    double tg[2];
    Tang(e, t, tg);
    out[0] = tg[1];
    out[1] = -tg[0];
  }
};

}  // namespace

std::string validate_instance(const HostInstance& h) {
  const int64_t C = h.C, E = h.E, N = h.N;
  if (C <= 0 || E <= 0 || N <= 0) return "mesh must have cells, edges and nodes";
  if (C > (1ll << 29) || E > (1ll << 30) || N > (1ll << 30)) return "mesh too large for int32 device indexing";
  for (int64_t e = 0; e < E; ++e) {
    int64_t a = h.en[2 * e], b = h.en[2 * e + 1];
    if (a < 0 || a >= N || b < 0 || b >= N || a == b) return "edge_nodes[" + std::to_string(e) + "] out of range";
    int64_t o = h.ec[2 * e], n = h.ec[2 * e + 1];
    if (o < 0 || o >= C) return "edge_cells[" + std::to_string(e) + "][0] out of range";
    if (n >= C) return "edge_cells[" + std::to_string(e) + "][1] out of range";
    if (n < -1)
      return "edge_cells[" + std::to_string(e) + "][1] = " + std::to_string(n) +
             ": only the solid-wall code -1 is implemented (Boundaries::SOLID_WALL)";
    if (n == o) return "edge_cells[" + std::to_string(e) + "] joins a cell to itself";
  }
  for (int64_t i = 0; i < C; ++i) {
    for (int k = 0; k < 3; ++k) {
      int64_t nd = h.cn[3 * i + k];
      if (nd < 0 || nd >= N) return "cell_nodes[" + std::to_string(i) + "] out of range";
      int64_t e = h.ce[3 * i + k];
      if (e < 0 || e >= E) return "cell_edges[" + std::to_string(i) + "] out of range";
      int64_t o = h.ec[2 * e], n = h.ec[2 * e + 1];
      int64_t nb = h.ct[3 * i + k];
      if (o == i) {
        if (nb != n) return "cell_neighbours[" + std::to_string(i) + "] disagrees with edge_cells";
      } else if (n == i) {
        if (nb != o) return "cell_neighbours[" + std::to_string(i) + "] disagrees with edge_cells";
      } else {
        return "cell " + std::to_string(i) + " lists edge " + std::to_string(e) + " that does not touch it";
      }
    }
    if (h.ce[3 * i] == h.ce[3 * i + 1] || h.ce[3 * i] == h.ce[3 * i + 2] || h.ce[3 * i + 1] == h.ce[3 * i + 2])
      return "cell " + std::to_string(i) + " lists an edge twice";
  }
  for (size_t q = 0; q < h.geom.size(); ++q)
    if (!std::isfinite(h.geom[q])) return "non-finite geometry";
  Geo g{h};
  for (int64_t i = 0; i < C; ++i)
    if (!(g.Area(i) > 0.)) return "cell " + std::to_string(i) + " has zero area";
  return "";
}

void precompute_instance(const HostInstance& h, int inst, int64_t c0, int64_t e0, int64_t n0, HostImage& img) {
  const int64_t C = h.C, E = h.E, N = h.N, Ct = img.C;
  Geo g{h};
  const double inf = std::numeric_limits<double>::infinity();
  img.inst_cell_begin[inst] = (int)c0;
  img.inst_cfl[inst] = h.cfl;
  img.inst_cor[inst] = h.cor;
  for (int64_t n = 0; n < N; ++n) img.nz[n0 + n] = h.geom[3 * n + 2];
  // the cells around each node, a CSR over this instance's nodes whose
  // entries start at 3 c0 (each cell has three nodes): PartWet2 gathers its
  // lowest node's maximum over them (src/MUSCLObject.cpp:138-140)
  {
    std::vector<int64_t> at((size_t)N + 1, 0);
    for (int64_t i = 0; i < 3 * C; ++i) at[h.cn[i] + 1]++;
    for (int64_t n = 0; n < N; ++n) at[n + 1] += at[n];
    for (int64_t n = 0; n <= N; ++n) img.nptr[n0 + n] = (int)(3 * c0 + at[n]);
    for (int64_t i = 0; i < C; ++i)
      for (int k = 0; k < 3; ++k) img.ncell[3 * c0 + at[h.cn[3 * i + k]]++] = (int)(((c0 + i) << 2) | k);
  }

  auto cell_range = [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      const int64_t gi = c0 + i;
      const int64_t* ip = h.cn.data() + 3 * i;
      const int64_t* ie = h.ce.data() + 3 * i;
      const int64_t* it = h.ct.data() + 3 * i;
      img.cinst[gi] = inst;
      unsigned char own = 0;
      bool boundary = false;
      for (int k = 0; k < 3; ++k) {
        img.cnode[k * Ct + gi] = (int)(n0 + ip[k]);
        img.cnbr[k * Ct + gi] = it[k] < 0 ? -1 : (int)(c0 + it[k]);
        img.cedge[k * Ct + gi] = (int)(e0 + ie[k]);
        if (h.ec[2 * ie[k]] == i) own |= (unsigned char)(1u << k);
        if (h.ec[2 * ie[k] + 1] < 0) boundary = true;  // src/TriangMesh.cpp:18-23
      }
      img.cown[gi] = own;
      double ti[3];
      g.T(i, ti);
      const double bci = ti[2];
      img.bc[gi] = bci;
      const double area = g.Area(i);
      img.area[gi] = area;
      const double* P0 = g.P(ip[0]);
      const double* P1 = g.P(ip[1]);
      const double* P2 = g.P(ip[2]);
      // src/MUSCLObject.cpp:17-25 (maxCoeff of the node z)
      double mx = P0[2];
      if (P1[2] > mx) mx = P1[2];
      if (P2[2] > mx) mx = P2[2];
      img.fwthr[gi] = boundary ? inf : mx;
      const double i_area = 1. / area;
      double Ek[3][3];
      for (int k = 0; k < 3; ++k) {
        img.zn[k * Ct + gi] = g.P(ip[k])[2];
        g.Emid(ie[k], Ek[k]);
        img.ze[k * Ct + gi] = Ek[k][2];
        img.cek[k * Ct + gi] = i_area * g.L(ie[k]);  // src/TimeDisc.cpp:17,28
        double nrm[2];
        g.Norm(ie[k], i, nrm);  // src/TimeDisc.cpp:35
        // n c: the pressure term's geometry factor (src/TimeDisc.cpp:35 evaluates
        // n(e, i) * c first), kept whole so the update multiplies once
        img.cnxc[k * Ct + gi] = nrm[0] * img.cek[k * Ct + gi];
        img.cnyc[k * Ct + gi] = nrm[1] * img.cek[k * Ct + gi];
        img.srec[k * Ct + gi] = SlotRec{img.cek[k * Ct + gi], img.ze[k * Ct + gi], img.cnxc[k * Ct + gi],
                                        img.cnyc[k * Ct + gi]};
        img.cslot[k * Ct + gi] = int2{img.cedge[k * Ct + gi], img.cnbr[k * Ct + gi]};
      }
      // ---- dry cell: ReconstructDryCell + UpdateInterfaceValues
      // (src/MUSCLObject.cpp:31-36, include/MUSCLObject.h:26-33, src/Assigners.cpp:8-20)
      double sx, sy;
      plane_gradient(P0[0], P0[1], P0[2], P1[0], P1[1], P1[2], P2[0], P2[1], P2[2], &sx, &sy);
      double* dr = img.dry.data() + (size_t)gi * kDryStride;
      for (int k = 0; k < 3; ++k) {
        const double* Pk = g.P(ip[k]);
        double a0 = bci + (sx * (Pk[0] - ti[0]) + sy * (Pk[1] - ti[1]));
        dr[k] = ((a0 - Pk[2]) >= 0) ? a0 : Pk[2];
        double e0v = bci + (sx * (Ek[k][0] - ti[0]) + sy * (Ek[k][1] - ti[1]));
        double at = ((e0v - Ek[k][2]) >= 0) ? e0v : Ek[k][2];
        double ow, ou, ov;
        prim_assign(Ek[k][2], at, 0., 0., &ow, &ou, &ov);
        dr[3 + k] = ow;
      }
      dr[6] = sx;
      dr[7] = sy;
      // ---- fully-wet cell planes for every wet/part-wet neighbour combination
      // (src/MUSCLObject.cpp:38-84); bit k set = neighbour k partially wet.
      if (!boundary) {
        double Tn[3][3];
        for (int k = 0; k < 3; ++k) g.T(it[k], Tn[k]);
        const double third = 1. / 3.;
        const double diag = 1. - third;
        double dxk[3][2];
        for (int k = 0; k < 3; ++k)
          for (int r = 0; r < 2; ++r) {
            double m0 = (k == 0) ? diag : -third;
            double m1 = (k == 1) ? diag : -third;
            double m2 = (k == 2) ? diag : -third;
            dxk[k][r] = P0[r] * m0 + P1[r] * m1 + P2[r] * m2;
          }
        for (int mask = 0; mask < 8; ++mask) {
          const double* pk[3];
          for (int k = 0; k < 3; ++k) pk[k] = (mask >> k & 1) ? Ek[k] : Tn[k];
          double g0, g1;
          plane_gradient(pk[0][0], pk[0][1], pk[0][2], pk[1][0], pk[1][1], pk[1][2], pk[2][0], pk[2][1], pk[2][2],
                         &g0, &g1);
          double* rec = img.combo.data() + combo_off((int)Ct, (int)gi, mask);
          rec[0] = g0;
          rec[1] = g1;
          for (int k = 0; k < 3; ++k) {
            rec[2 + k] = g0 * dxk[k][0] + g1 * dxk[k][1];                            // positivity offsets
            rec[5 + k] = g0 * (Ek[k][0] - ti[0]) + g1 * (Ek[k][1] - ti[1]);          // edge-centre offsets
            const double* Pk = g.P(ip[k]);
            rec[8 + k] = g0 * (Pk[0] - ti[0]) + g1 * (Pk[1] - ti[1]);                // vertex offsets
          }
          rec[11] = 0.;
        }
      }
      // ---- PartWet1 (src/MUSCLObject.cpp:86-112)
      {
        double z0 = P0[2], z1 = P1[2], z2 = P2[2];
        double b13 = z0, b23 = z0;
        if (z1 > b13) b13 = z1;
        if (z2 > b13) b13 = z2;
        if (z1 < b23) b23 = z1;
        if (z2 < b23) b23 = z2;
        double b12 = 3. * bci - b23 - b13;
        double* p = img.pw1.data() + (size_t)gi * kPw1Stride;
        p[0] = b13;
        p[1] = b23;
        p[2] = b12;
        p[3] = b12 + (1. / 3.) * (b13 - b12) * (b13 - b12) / (b13 - b23);  // b_delimiter
        p[4] = -3. * b13;                                                     // cubic b
        p[5] = 3. * (b12 * b13 + b13 * b23 - b12 * b23);                      // cubic c
        p[6] = b13 - b23;
        p[7] = b12 - b23;
        p[8] = b13 - b12;
        p[9] = b12 * (b12 + b23);
        p[10] = b23 * b23 * b13;
        p[11] = 0.;
      }
      // ---- PartWet2 (src/MUSCLObject.cpp:114-191)
      {
        int64_t sp[3] = {ip[0], ip[1], ip[2]};
        int64_t t;
        if (g.P(sp[0])[2] > g.P(sp[1])[2]) { t = sp[0]; sp[0] = sp[1]; sp[1] = t; }
        if (g.P(sp[1])[2] > g.P(sp[2])[2]) { t = sp[1]; sp[1] = sp[2]; sp[2] = t; }
        if (g.P(sp[0])[2] > g.P(sp[1])[2]) { t = sp[0]; sp[0] = sp[1]; sp[1] = t; }
        Pw2Rec& q = img.pw2[gi];
        for (int k = 0; k < 3; ++k)
          for (int r = 0; r < 3; ++r) q.p[k][r] = g.P(sp[k])[r];
        double b23 = q.p[0][2], b12 = q.p[1][2], b13 = q.p[2][2];
        q.flat = (b13 - b23 < kTol) ? 1 : 0;
        q.ratio_b = (b12 - b23) / (b13 - b23);
        q.hd2f = 2. * b13 - b12 - b23;
        q.d13 = b13 - b23;
        q.beta = (b13 - b12) / (b13 - b23);
        q.tp0x = ti[0] - q.p[0][0];
        q.tp0y = ti[1] - q.p[0][1];
        for (int k = 0; k < 3; ++k) {
          const double* Pk = g.P(ip[k]);
          q.dnode[k][0] = Pk[0] - ti[0];
          q.dnode[k][1] = Pk[1] - ti[1];
          q.dedge[k][0] = Ek[k][0] - ti[0];
          q.dedge[k][1] = Ek[k][1] - ti[1];
        }
        q.lo = (int)(n0 + sp[0]);
        for (int s2 = 0; s2 < 3; ++s2)
          for (int k = 0; k < 3; ++k)
            if (ip[k] == sp[s2]) q.sk[s2] = k;
        q.pad = 0;
      }
    }
  };

  auto edge_range = [&](int64_t lo, int64_t hi) {
    for (int64_t e = lo; e < hi; ++e) {
      const int64_t ge = e0 + e;
      int64_t o = h.ec[2 * e], n = h.ec[2 * e + 1];
      img.einst[ge] = inst;
      img.eown[ge] = (int)(c0 + o);
      img.enb[ge] = n < 0 ? -1 : (int)(c0 + n);
      int ko = 0, kn = 0;
      for (int k = 0; k < 3; ++k) {
        if (h.ce[3 * o + k] == e) ko = k;
        if (n >= 0 && h.ce[3 * n + k] == e) kn = k;
      }
      img.eslotl[ge] = (int)(ko * Ct + c0 + o);
      img.eslotr[ge] = n < 0 ? -1 : (int)(kn * Ct + c0 + n);
      double nrm[2], tg[2], em[3];
      g.Norm(e, o, nrm);
      g.Tang(e, o, tg);
      g.Emid(e, em);
      img.enx[ge] = nrm[0];
      img.eny[ge] = nrm[1];
      img.etx[ge] = tg[0];
      img.ety[ge] = tg[1];
      img.ezm[ge] = em[2];
      if (n >= 0) {
        double L = g.L(e);
        double dl = 2. * g.Area(o) / L;  // include/Fluxes.h:43-44, 86-87
        double dr = 2. * g.Area(n) / L;
        img.elmin[ge] = smin(dl, dr);
      } else {
        img.elmin[ge] = 0.;
      }
      img.erec[ge] = EdgeRec{img.enx[ge], img.eny[ge], img.etx[ge], img.ety[ge], img.ezm[ge], img.elmin[ge]};
      img.eidx[ge] = int4{img.eown[ge], img.enb[ge], img.eslotl[ge], img.eslotr[ge]};
    }
  };

  unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (C + E < 20000) nt = 1;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t) {
    int64_t clo = C * t / nt, chi = C * (t + 1) / nt;
    int64_t elo = E * t / nt, ehi = E * (t + 1) / nt;
    th.emplace_back([=, &cell_range, &edge_range] {
      cell_range(clo, chi);
      edge_range(elo, ehi);
    });
  }
  for (auto& x : th) x.join();
}

}  // namespace swe
