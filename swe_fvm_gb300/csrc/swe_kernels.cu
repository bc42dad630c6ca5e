// swe_kernels.cu -- sm_103a kernels of one Runge-Kutta stage and the engine
// that sequences them.
//
// A stage (src/Solvers.cpp:5-59) is six kernels over the concatenated cells
// and edges of every instance:
//   k_recon1  all cells    SpaceDisc::ComputeInterfaceValues pass 1
//                          (src/SpaceDisc.cpp:37-45), listing the partially
//                          wet cells
//   k_recon2  part-wet     pass 2 (src/SpaceDisc.cpp:47-51), gathering the
//                          node maximum it reads from the pass-1 values of
//                          the node's cells (order-independent)
//   k_flux    all edges    SpaceDisc::ComputeFluxes (src/SpaceDisc.cpp:54-74)
//                          with the flux plugin and the CFL min-reduction,
//                          except the edges of partially-wet cells
//   k_flux_pw those edges  on a second stream, after k_recon2
//   k_drain   all cells    TimeDisc::ComputeDrainingDt (src/TimeDisc.cpp:43-66),
//                          once per cell instead of 4x per RHS
//   k_update  all cells    TimeDisc::RHS + ConsAssigner (src/TimeDisc.cpp:3-41,
//                          src/Assigners.cpp:28-44), an edge-to-cell gather
// Every read of a stage comes from the start-of-stage state, so results do not
// depend on the cell order or on scheduling; the only atomics (CFL minimum,
// part-wet list append) are exact min/append operations.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>

#include "swe_engine.cuh"

namespace swe {

Scheme scheme_table(int scheme) {
  Scheme s{};
  s.s[0] = Stage{true, 0., 0., 1.};
  if (scheme == 0) {
    s.n = 1;
  } else if (scheme == 1) {
    s.n = 2;
    s.s[1] = Stage{false, 0.5, 0.5, 0.5};
  } else {
    s.n = 3;
    s.s[1] = Stage{false, 0.75, 0.25, 0.25};
    s.s[2] = Stage{false, 1. / 3., 2. / 3., 2. / 3.};
  }
  return s;
}

namespace {

constexpr double kInf = __builtin_huge_val();

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// start moving the cache line of p towards this SM's L1 (no register, no wait)
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// two 16-byte loads of a 32-byte record through the read-only path
__device__ __forceinline__ void ldg_pair(const void* p, double2* a, double2* b) {
  const double2* q = (const double2*)p;
  *a = __ldg(q);
  *b = __ldg(q + 1);
}

// ------------------------------------------------------------ interface write
// UpdateInterfaceValues for one edge slot (src/SpaceDisc.cpp:24-29): AtPoint
// value (w, u, v) already dry-checked, through PrimAssigner with the edge
// bathymetry, plus the source gradient and Coriolis term.
// Source gradient plus the Coriolis term, (gx, gy) + cor (-v, u).  COR0 (cor
// is +-0 for every instance): x + (+-0) is x unless x is itself a zero, and
// then -0 only if both are -0, so the same bits come from integer operations.
// (A non-finite velocity would give NaN through the arithmetic; its state is
// already non-finite and reported by the update kernel.)
__device__ __forceinline__ double add_zero_product(double x, double c, double v) {
  const unsigned long long ux = (unsigned long long)dbits(x);
  if ((ux << 1) != 0ull) return x;
  const unsigned long long uc = (unsigned long long)dbits(c);
  const unsigned long long uv = (unsigned long long)dbits(v);
  return dfrom((long long)(ux & (uc ^ uv) & 0x8000000000000000ull));
}

template <bool COR0>
__device__ __forceinline__ void write_slot(const DevWork& wk, int slot, double be, double w, double u, double v,
                                           double gx, double gy, double cor) {
  double ow, ou, ov;
  prim_assign(be, w, u, v, &ow, &ou, &ov);
  wk.ew[slot] = ow;
  wk.eu[slot] = ou;
  wk.ev[slot] = ov;
  double sx = gx, sy = gy;
  if (COR0) {
    const double nov = dfrom(dbits(ov) ^ (long long)0x8000000000000000ull);
    sx = add_zero_product(gx, cor, nov);
    sy = add_zero_product(gy, cor, ou);
  } else {
    sx += cor * (-ov);
    sy += cor * ou;
  }
  wk.sx[slot] = sx;
  wk.sy[slot] = sy;
}

// MUSCL::AtPoint with a w-only plane (include/MUSCLObject.h:26-33): the value
// at a point whose offset term is `off` and whose bathymetry is z.
__device__ __forceinline__ bool at_point_wet(double w0, double off, double z, double* wout) {
  double a = w0 + off;
  if (dge0(a - z)) {
    *wout = a;
    return true;
  }
  *wout = z;
  return false;
}

// Pass-1 AtPoint value of cell c at its local node kn, from what pass 1 left:
// the class byte (dry / partially wet / fully wet, combination mask, plane
// kept), the PartWet1 level of a partially-wet cell and the state.
__device__ __forceinline__ double pass1_value(const DevMesh& m, const DevWork& wk, const double* __restrict__ W,
                                              int c, int kn) {
  const int C = m.C;
  const unsigned cl = wk.cls[c];
  if ((cl & 3u) == 0u) return m.dry[(size_t)c * kDryStride + kn];
  const double z = m.zn[kn * C + c];
  double val;
  if ((cl & 3u) == 1u) {
    at_point_wet(wk.pwrec[c], 0., z, &val);  // the PartWet1 level, a flat plane
  } else {
    // the combination plane's vertex offset when pass 1 kept the plane, else flat
    const double off = (cl & 32u) ? m.combo[combo_off(C, c, (int)((cl >> 2) & 7u)) + 8 + kn] : 0.;
    at_point_wet(W[c], off, z, &val);
  }
  return val;
}

// The node maximum m_max_wp of node nd (src/MUSCLObject.cpp:13-36): the
// largest pass-1 AtPoint value of the cells around it, starting from the
// node's bathymetry (every AtPoint value is >= it).  A maximum is exact and
// order-free, so gathering it where it is needed gives the value the
// reference's accumulation over its cell loop gives.
__device__ __forceinline__ unsigned long long node_max_key(const DevMesh& m, const DevWork& wk,
                                                           const double* __restrict__ W, int nd) {
  unsigned long long key = order_key(m.nz[nd]);
  const int q0 = m.nptr[nd], q1 = m.nptr[nd + 1];
  // the first 8 cells (a triangulation node has about 6) with their loads
  // issued together, the rest one by one
  constexpr int kV = 8;
  int cq[kV];
#pragma unroll
  for (int j = 0; j < kV; ++j) cq[j] = q0 + j < q1 ? m.ncell[gidx(wk, q0 + j, 3 * m.C)] : -1;
#pragma unroll
  for (int j = 0; j < kV; ++j) {
    if (cq[j] >= 0) {
      const unsigned long long k = order_key(pass1_value(m, wk, W, gidx(wk, cq[j] >> 2, m.C), cq[j] & 3));
      key = k > key ? k : key;
    }
  }
  for (int q = q0 + kV; q < q1; ++q) {
    const int c = m.ncell[gidx(wk, q, 3 * m.C)];
    const unsigned long long k = order_key(pass1_value(m, wk, W, gidx(wk, c >> 2, m.C), c & 3));
    key = k > key ? k : key;
  }
  return key;
}

// PartWet1 level (src/MUSCLObject.cpp:86-112)
__device__ __forceinline__ double partwet1_level(const double* __restrict__ p, double w, double h) {
  const double b13 = p[0], b23 = p[1], b12 = p[2], bdel = p[3];
  if (dle(b13, w)) return w;
  if (dle(w, bdel)) return b23 + cbrt_rn(3. * h * p[6] * p[7]);
  double cc = p[6] * (3. * h * p[8] - p[9]) - p[10];
  (void)b12;
  return bisection(cc, p[5], p[4], p[2], b13);
}

// ---------------------------------------------------------------- kernels
template <bool BATCH, bool COR0>
__global__ void __launch_bounds__(256, 5) k_recon1(DevMesh m, DevWork wk, const double* __restrict__ W,
                                                const double* __restrict__ U, const double* __restrict__ V,
                                                int latch_mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool part = false;
  unsigned char cls = 0;  // dry unless set below
  if (i < m.C) {
    const int inst = BATCH ? m.cinst[i] : 0;
    if (i == (BATCH ? m.inst_cell_begin[inst] : 0)) {
      if (latch_mode == 1) {  // dt = TimeDisc::CFLdt() of the previous flux pass
        double dt = m.inst_cfl[inst] * order_val(wk.r[inst]);
        wk.dt[inst] = dt;
        wk.tsum[inst] += dt;
      } else if (latch_mode == 2) {
        double dt = wk.fixed_dt[BATCH ? inst : 0];
        wk.dt[inst] = dt;
        wk.tsum[inst] += dt;
      }
      wk.r[inst] = order_key(1.0);  // src/SpaceDisc.cpp:56
    }
    const int C = m.C;
    // the combination record of the all-fully-wet neighbourhood (mask 0) is
    // the one nearly every fully-wet cell reads: start its lines towards L1
    // now, before the loads that decide the class and the mask
    prefetch_l1(m.combo + combo_off(C, i, 0));
    prefetch_l1(m.combo + combo_off(C, i, 0) + 8);
    const double cor = m.inst_cor[inst];
    const double w = W[i], u = U[i], v = V[i];
    const double h = w - m.bc[i];
    if (!is_wet(h)) {
      // ReconstructDryCell: every value is a mesh constant
      const double* dr = m.dry + (size_t)i * kDryStride;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int slot = k * C + i;
        write_slot<COR0>(wk, slot, m.ze[slot], dr[3 + k], 0., 0., dr[6], dr[7], cor);
      }
    } else if (!dlt(m.fwthr[i], w)) {
      // partially wet: the PartWet1 level now, PartWet2 in k_recon2
      wk.pwrec[i] = partwet1_level(m.pw1 + (size_t)i * kPw1Stride, w, h);
      part = true;
      cls = 1;
    } else {
      // ReconstructFullWetCell (src/MUSCLObject.cpp:38-84)
      int mask = 0;
      bool first_order = false;
      double wn[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int nb = gidx(wk, m.cnbr[k * C + i], C);  // never a wall: fully-wet cells are interior
        const double wj = W[nb];
        wn[k] = wj;
        if (dlt(m.fwthr[nb], wj)) {
          // fully-wet neighbour: plane point at its centroid
        } else if (!is_wet(wj - m.bc[nb])) {
          first_order = true;
        } else {
          mask |= 1 << k;  // partially-wet neighbour: plane point at the edge centre
        }
      }
      cls = (unsigned char)(2 | (mask << 2));
      double gx = 0., gy = 0.;
      double toff[3] = {0., 0., 0.};
      if (!first_order) {
        const double* rec = m.combo + combo_off(C, i, mask);
        const double g0 = rec[0], g1 = rec[1];
        bool pos = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const double hp = (rec[2 + k] + w) - m.zn[k * C + i];
          if (!is_wet(hp)) pos = false;
        }
        if (pos) {
          // binary TVD limiter on the w row (rows u, v of df are zero)
          bool tvd = true;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const double vmin = smin(w, wn[k]), vmax = smax(w, wn[k]);
            const double vek = w + rec[5 + k];
            if (!(dle(vmin, vek) && dle(vek, vmax))) tvd = false;
          }
          if (tvd) {
            cls |= 32;  // combination plane kept
            gx = g0;
            gy = g1;
#pragma unroll
            for (int k = 0; k < 3; ++k) toff[k] = rec[5 + k];
          } else {
            gx = 0. * g0;  // diag(TVD) * df keeps the sign of zero
            gy = 0. * g1;
          }
        }
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int slot = k * C + i;
        const double be = m.ze[slot];
        double we;
        if (at_point_wet(w, toff[k], be, &we)) write_slot<COR0>(wk, slot, be, we, u, v, gx, gy, cor);
        else write_slot<COR0>(wk, slot, be, we, 0., 0., gx, gy, cor);
      }
    }
  }
  if (i < m.C) wk.cls[i] = cls;
  // warp-aggregated append of the partially-wet cells
  const unsigned bal = __ballot_sync(0xffffffffu, part);
  if (bal) {
    const int leader = __ffs(bal) - 1;
    int base = 0;
    if (lane_id() == leader) base = atomicAdd(wk.pwcount, __popc(bal));
    base = __shfl_sync(0xffffffffu, base, leader);
    const int slot = base + __popc(bal & ((1u << lane_id()) - 1u));
    if (part && slot < m.C) wk.pwlist[slot] = i;
  }
}

// Every node maximum (the reference's m_max_wp after pass 1), for the
// interface-value entry points that return them; the step itself gathers
// only the nodes PartWet2 reads (k_recon2).
__global__ void k_node_max_all(DevMesh m, DevWork wk, const double* __restrict__ W) {
  const int nd = blockIdx.x * blockDim.x + threadIdx.x;
  if (nd < m.N) wk.maxwp[nd] = node_max_key(m, wk, W, nd);
}

// ReconstructPartWetCell2 (src/MUSCLObject.cpp:114-191) over the listed cells.
template <bool BATCH, bool COR0>
__global__ void __launch_bounds__(256) k_recon2(DevMesh m, DevWork wk, const double* __restrict__ W,
                                                const double* __restrict__ U, const double* __restrict__ V) {
  const int C = m.C;
  const int n = min(*wk.pwcount, C);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int i = gidx(wk, wk.pwlist[q], C);
    const int inst = BATCH ? m.cinst[i] : 0;
    const double cor = m.inst_cor[inst];
    const double w = W[i], u = U[i], v = V[i];
    const Pw2Rec& r = m.pw2[i];
    const double b23 = r.p[0][2], b12 = r.p[1][2], b13 = r.p[2][2];
    double w0 = wk.pwrec[i];  // PartWet1 fallback level
    double gx = 0., gy = 0.;
    bool plane = false;
    if (!(dlt(b13, w) || r.flat)) {
      // the node maximum of the lowest node, gathered from its cells' pass-1
      // values; kept in maxwp for the adjoint's reverse of this cell
      const int lo = gidx(wk, r.lo, m.N);
      const unsigned long long key = node_max_key(m, wk, W, lo);
      wk.maxwp[lo] = key;
      const double w23 = order_val(key);
      const double h23 = w23 - b23;
      const double ratio_b = r.ratio_b;
      const double h_delim1 = 1. / 3. * h23 * ratio_b;
      const double h_delim2 = SWE_DIV(1. / 3. * h23 * r.hd2f, r.d13);
      const double hi = w - m.bc[i];
      const double ratio_h = SWE_DIV(hi, h23);
      // columns of the reference's `points` after all its writes: point 0 is
      // the lowest vertex with its bathymetry (see the restatement's notes)
      double p1x, p1y, p1z, p2x, p2y, p2z;
      bool ok = true;
      if (dle(hi, h_delim1)) {
        const double k2 = SWE_SQRT(SWE_DIV(3. * ratio_h, ratio_b));
        p1x = k2 * r.p[1][0] + (1. - k2) * r.p[0][0];
        p1y = k2 * r.p[1][1] + (1. - k2) * r.p[0][1];
        p1z = k2 * r.p[1][2] + (1. - k2) * r.p[0][2];
        const double k3 = SWE_SQRT(3. * ratio_h * ratio_b);
        p2x = k3 * r.p[2][0] + (1. - k3) * r.p[0][0];
        p2y = k3 * r.p[2][1] + (1. - k3) * r.p[0][1];
        p2z = k3 * r.p[2][2] + (1. - k3) * r.p[0][2];
      } else if (dle(h_delim2, hi)) {
        const double delta_w = 1.5 * (hi - h_delim2);
        p1x = r.p[1][0]; p1y = r.p[1][1]; p1z = r.p[1][2];
        p2x = r.p[2][0]; p2y = r.p[2][1]; p2z = r.p[2][2];
        p2z += delta_w;
      } else {
        const double alpha = 3. * ratio_h;
        const double beta = r.beta;
        const double k1 = 1. - bisection(SWE_DIV(1. + beta - alpha, beta * beta), SWE_DIV(alpha - 3., beta), 0., 0., 1.);
        if (dltc(k1, kTol)) {
          ok = false;
        } else {
          const double bp1 = k1 * b13 + (1. - k1) * b12;
          p1x = r.p[1][0]; p1y = r.p[1][1]; p1z = r.p[1][2];
          p2x = k1 * r.p[2][0] + (1. - k1) * r.p[1][0];
          p2y = k1 * r.p[2][1] + (1. - k1) * r.p[1][1];
          p2z = bp1;
        }
      }
      if (ok) {
        plane_gradient(r.p[0][0], r.p[0][1], r.p[0][2], p1x, p1y, p1z, p2x, p2y, p2z, &gx, &gy);
        w0 = w23 + (gx * r.tp0x + gy * r.tp0y);
        plane = true;
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int slot = k * C + i;
      const double be = m.ze[slot];
      const double off = plane ? (gx * r.dedge[k][0] + gy * r.dedge[k][1]) : 0.;
      double we;
      if (at_point_wet(w0, off, be, &we)) write_slot<COR0>(wk, slot, be, we, u, v, gx, gy, cor);
      else write_slot<COR0>(wk, slot, be, we, 0., 0., gx, gy, cor);
    }
  }
}

// SpaceDisc::ComputeFluxes with flux plugin FLUX and the CFL min-reduction.
// The flux of edge e (src/SpaceDisc.cpp:54-74) into f0..f2; *lw receives its
// length-to-wavespeed ratio or stays +inf.
template <class FLUX, bool TAPE>
__device__ __forceinline__ void flux_edge(const DevMesh& m, const DevWork& wk, const double* __restrict__ W, int e,
                                          int inst, double* lw) {
  const int4 ix = __ldg(m.eidx + e);  // (owner, neighbour, owner's slot, neighbour's slot)
  const int o = gidx(wk, ix.x, m.C);
  const int nb = ix.y;
  double F[3];
  const double2* gr = (const double2*)(m.erec + e);
  const double2 n2 = __ldg(gr);
  const double nx = n2.x, ny = n2.y;
  if (nb < 0) {
    // solid wall: ElemFlux with the owner's cell-average depth (src/SpaceDisc.cpp:66-69)
    elem_flux(nx, ny, W[o] - m.bc[o], 0., 0., F);
  } else {
    const double2 t2 = __ldg(gr + 1), bl = __ldg(gr + 2);
    EdgeGeom g;
    g.nx = nx; g.ny = ny;
    g.tx = t2.x; g.ty = t2.y;
    g.b = bl.x;
    g.lmin = bl.y;
    const int sl = gidx(wk, ix.z, 3 * m.C), sr = gidx(wk, ix.w, 3 * m.C);
    SideState L{wk.ew[sl], wk.eu[sl], wk.ev[sl]};
    SideState R{wk.ew[sr], wk.eu[sr], wk.ev[sr]};
    if (TAPE) FLUX::eval(g, L, R, m.inst_cor[inst], lw, F, EdgeTape{wk.ftape, m.E, e});
    else FLUX::eval(g, L, R, m.inst_cor[inst], lw, F);
  }
  wk.f0[e] = F[0];
  wk.f1[e] = F[1];
  wk.f2[e] = F[2];
}

// MODE 0: every edge.  MODE 1: the edges none of whose cells is partially
// wet (the others wait for PartWet2 and go through k_flux_pw).
// TAPE: also store the intermediates the adjoint's reverse reads (wk.ftape).
// Register caps (the second __launch_bounds__ argument: blocks of 256 threads
// per SM) measured on the 1M-cell dam break, CUDA events, same bits: k_flux at
// 64 registers 0.211 -> 0.199 ms per launch, k_recon1 at 48 registers
// 0.091 -> 0.087 ms; more resident warps hide the gathers better than the
// few spilled registers cost.
template <class FLUX, bool BATCH, int MODE, bool TAPE>
__global__ void __launch_bounds__(256, 4) k_flux(DevMesh m, DevWork wk, const double* __restrict__ W) {
  __shared__ unsigned long long s_min[32];
  __shared__ int s_inst[32];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  double lw = kInf;
  int inst = 0;
  if (e < m.E) {
    if (BATCH) inst = m.einst[e];
    bool mine = true;
    if (MODE == 1) {
      const int nb = m.enb[e];
      mine = !(((wk.cls[gidx(wk, m.eown[e], m.C)] & 3) == 1) || (nb >= 0 && (wk.cls[gidx(wk, nb, m.C)] & 3) == 1));
    }
    if (mine) flux_edge<FLUX, TAPE>(m, wk, W, e, inst, &lw);
  }
  // min-reduction of the length-to-wavespeed ratio on order-preserving integer
  // keys (exact): warp, block, one atomicMin per block and instance
  const unsigned long long kNone = ~0ull;
  unsigned long long key = (dbits(lw) == dbits(kInf)) ? kNone : order_key(lw);
  const int lane = lane_id(), warp = threadIdx.x >> 5;
  const int inst0 = __shfl_sync(0xffffffffu, inst, 0);
  const bool warp_uniform = __all_sync(0xffffffffu, inst == inst0);
  if (warp_uniform) {
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const unsigned long long o = __shfl_xor_sync(0xffffffffu, key, off);
      key = o < key ? o : key;
    }
    if (lane == 0) {
      s_min[warp] = key;
      s_inst[warp] = inst0;
    }
  } else {
    if (key != kNone) atomicMin(wk.r + inst, key);
    if (lane == 0) {
      s_min[warp] = kNone;
      s_inst[warp] = -1;
    }
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    unsigned long long v = lane < nw ? s_min[lane] : kNone;
    int vi = lane < nw ? s_inst[lane] : s_inst[0];
    const int vi0 = __shfl_sync(0xffffffffu, vi, 0);
    const bool uni = __all_sync(0xffffffffu, vi == vi0 || v == kNone);
    if (uni) {
#pragma unroll
      for (int off = 16; off; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, off);
        v = o < v ? o : v;
      }
      if (lane == 0 && v != kNone) atomicMin(wk.r + vi0, v);
    } else if (v != kNone && vi >= 0) {
      atomicMin(wk.r + vi, v);
    }
  }
}

// The fluxes of the edges next to the stage's partially-wet cells (after
// PartWet2): listed cell i takes its local edge k unless the edge's owner is
// partially wet too and is not i, so that each edge is evaluated once.
template <class FLUX, bool BATCH, bool TAPE>
__global__ void __launch_bounds__(128) k_flux_pw(DevMesh m, DevWork wk, const double* __restrict__ W) {
  const int C = m.C;
  const int n = 3 * min(*wk.pwcount, C);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int q = t / 3, k = t - 3 * q;
    const int i = gidx(wk, wk.pwlist[q], C);
    const int e = gidx(wk, m.cedge[k * C + i], m.E);
    const int o = gidx(wk, m.eown[e], C);
    if ((((wk.cls[o] & 3) == 1) ? o : m.enb[e]) != i) continue;
    const int inst = BATCH ? m.einst[e] : 0;
    double lw = kInf;
    flux_edge<FLUX, TAPE>(m, wk, W, e, inst, &lw);
    if (dbits(lw) != dbits(kInf)) atomicMin(wk.r + inst, order_key(lw));
  }
}

// TimeDisc::ComputeDrainingDt once per cell; also empties the part-wet list
// for the next reconstruction.
__global__ void __launch_bounds__(256) k_drain(DevMesh m, DevWork wk, const double* __restrict__ W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *wk.pwcount = 0;
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
      const double f = wk.f0[gidx(wk, m.cedge[k * m.C + i], m.E)];
      sum += smax(0., ((own >> k) & 1u) ? f : -f);
    }
    d = dgtc(sum, kTol) ? SWE_DIV(m.area[i] * h, sum) : kInf;
  }
  wk.drain[i] = d;
}

// TimeDisc::RHS + the Shu-Osher combination + ConsAssigner.
// The output may be the same array as Wp or W0 (in-place stages): each thread
// reads its own cell before writing it, so no pointer here is __restrict__.
// STORE_N also writes the state before ConsAssigner to nst [3][C] (for the
// adjoint's segment recompute).
// HALF: a stage with a = b = c = 1/2 (SSPRK2's second), whose products with
// the coefficients are exact halvings.
template <bool BATCH, bool STORE_N, bool HALF>
__global__ void __launch_bounds__(256, 5) k_update(DevMesh m, DevWork wk, const double* Wp, const double* Up,
                                                const double* Vp, const double* W0, const double* U0,
                                                const double* V0, double* Wo, double* Uo, double* Vo, Stage st,
                                                double* nst = nullptr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m.C) return;
  const int C = m.C;
  const int inst = BATCH ? m.cinst[i] : 0;
  const double dt = HALF ? SWE_HALF(wk.dt[inst]) : (st.first ? wk.dt[inst] : st.c * wk.dt[inst]);
  const unsigned own = m.cown[i];
  const double dti = wk.drain[i];
  double r0 = 0., r1 = 0., r2 = 0.;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int slot = k * C + i;
    const int2 en = __ldg(m.cslot + slot);  // (edge, neighbour)
    double2 ce, nc;                         // (L/A, edge-centre z), (n_x L/A, n_y L/A)
    ldg_pair(m.srec + slot, &ce, &nc);
    const int e = gidx(wk, en.x, m.E);
    // sgn = +1 for the edge's owner, else -1: products with it are sign changes
    const bool out = (own >> k) & 1u;
    const double F0 = wk.f0[e], F1 = wk.f1[e], F2 = wk.f2[e];
    const int nb = en.y;
    const double dtik = nb < 0 ? kInf : wk.drain[gidx(wk, nb, C)];
    const double dtk = (out ? dgt0(F0) : dlt(F0, 0.)) ? smin(dt, dti) : smin(dt, dtik);  // sgn F0 > 0
    const double c_ek = ce.x;
    const double h_ek = wk.ew[slot] - ce.y;
    const double s = (out ? dtk : SWE_NEG(dtk)) * c_ek;
    r0 -= s * F0;
    r1 -= s * F1;
    r2 -= s * F2;
    const double q = dt * (1. / 3.);
    r1 -= q * wk.sx[slot] * h_ek;
    r2 -= q * wk.sy[slot] * h_ek;
    const double p = SWE_HALF(h_ek) * h_ek;  // 0.5 h h
    r1 += dtk * (nc.x * p);  // (n_x c) p
    r2 += dtk * (nc.y * p);
  }
  const double b = m.bc[i];
  const double h0 = W0[i] - b;
  const double c00 = h0, c01 = h0 * U0[i], c02 = h0 * V0[i];
  double n0, n1, n2;
  if (st.first && !HALF) {
    n0 = c00 + r0;
    n1 = c01 + r1;
    n2 = c02 + r2;
  } else {
    const double hp = Wp[i] - b;
    const double c10 = hp, c11 = hp * Up[i], c12 = hp * Vp[i];
    if (HALF) {
      n0 = SWE_HALF(c00) + SWE_HALF(c10) + r0;
      n1 = SWE_HALF(c01) + SWE_HALF(c11) + r1;
      n2 = SWE_HALF(c02) + SWE_HALF(c12) + r2;
    } else {
      n0 = st.a * c00 + st.b * c10 + r0;
      n1 = st.a * c01 + st.b * c11 + r1;
      n2 = st.a * c02 + st.b * c12 + r2;
    }
  }
  if (STORE_N) {
    nst[i] = n0;
    nst[C + i] = n1;
    nst[2 * C + i] = n2;
  }
  double ow, ou, ov;
  cons_assign(b, n0, n1, n2, &ow, &ou, &ov);
  Wo[i] = ow;
  Uo[i] = ou;
  Vo[i] = ov;
  // non-finite check on the exponent bits (integer pipe)
  const unsigned long long xw = (unsigned long long)dbits(ow) >> 52,
                           xu = (unsigned long long)dbits(ou) >> 52,
                           xv = (unsigned long long)dbits(ov) >> 52;
  if (((xw & 0x7FFull) == 0x7FFull) || ((xu & 0x7FFull) == 0x7FFull) || ((xv & 0x7FFull) == 0x7FFull))
    atomicOr(wk.err, kErrNonFinite);
}

__global__ void k_init_nodes(DevMesh m, DevWork wk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m.N) wk.maxwp[i] = order_key(m.nz[i]);
  if (i == 0) *wk.pwcount = 0;
}

inline int nblocks(int64_t n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

// ------------------------------------------------------------------ engine
template <class T>
T* Engine::dalloc(size_t n) {
  void* p = nullptr;
  if (n == 0) n = 1;
  if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) return nullptr;
  allocs_.push_back(p);
  bytes_ += n * sizeof(T);
  return (T*)p;
}

void Engine::set_stream(cudaStream_t s) {
  cudaStream_t next = s ? s : own_stream_;
  if (next == stream_) return;
  cudaEvent_t ev = nullptr;
  if (stream_ && cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess) {
    if (cudaEventRecord(ev, stream_) == cudaSuccess) cudaStreamWaitEvent(next, ev, 0);
    cudaEventDestroy(ev);  // released once the wait is satisfied
  } else if (stream_) {
    cudaStreamSynchronize(stream_);
  }
  stream_ = next;
}

Engine::~Engine() {
  // nothing of this engine may still run on its own streams when its memory
  // goes (a caller's stream is synchronised by swe_destroy)
  if (own_stream_) cudaStreamSynchronize(own_stream_);
  if (side_) cudaStreamSynchronize(side_);
  if (adj_) adjoint_state_delete(adj_);
  for (auto& row : graphs_)
    for (auto& g : row)
      if (g) cudaGraphExecDestroy(g);
  for (void* p : allocs_) cudaFree(p);
  if (h_fixed_dt) cudaFreeHost(h_fixed_dt);
  if (own_stream_) cudaStreamDestroy(own_stream_);
  if (side_) cudaStreamDestroy(side_);
  if (ev_fork_) cudaEventDestroy(ev_fork_);
  if (ev_join_) cudaEventDestroy(ev_join_);
}

std::string Engine::init(std::vector<HostInstance>&& inst, int flux, int ws, int block, int* st, bool batched) {
  *st = 0;
  flux_ = flux;
  ws_ = ws;
  if (block > 0) blk_[0] = blk_[1] = blk_[2] = block;
  batched_ = batched;
  const int I = (int)inst.size();
  int64_t C = 0, E = 0, N = 0;
  cell_off.assign(I + 1, 0);
  edge_off.assign(I + 1, 0);
  node_off.assign(I + 1, 0);
  for (int q = 0; q < I; ++q) {
    std::string err = validate_instance(inst[q]);
    if (!err.empty()) {
      *st = 2;
      return (I > 1 ? "instance " + std::to_string(q) + ": " : std::string()) + err;
    }
    cell_off[q] = C;
    edge_off[q] = E;
    node_off[q] = N;
    C += inst[q].C;
    E += inst[q].E;
    N += inst[q].N;
  }
  cell_off[I] = C;
  edge_off[I] = E;
  node_off[I] = N;
  cor0_ = true;
  for (const auto& q : inst) cor0_ = cor0_ && q.cor == 0.;
  if (3 * C > (1ll << 31) - 1 || E > (1ll << 31) - 1 || N > (1ll << 31) - 1) {
    *st = 1;
    return "total mesh too large for int32 device indexing";
  }
  HostImage img;
  img.resize((int)C, (int)E, (int)N, I);
  for (int q = 0; q < I; ++q) precompute_instance(inst[q], q, cell_off[q], edge_off[q], node_off[q], img);

  // every mesh array is recorded (device pointer, bytes) in upload order, so
  // that set_bathymetry can refill the same buffers
  mesh_arrays_.clear();
  auto up = [&](auto& vec, auto*& dst) -> bool {
    using T = typename std::remove_reference<decltype(vec)>::type::value_type;
    T* d = dalloc<T>(vec.size());
    if (!d) return false;
    if (cudaMemcpy(d, vec.data(), vec.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    dst = d;
    mesh_arrays_.push_back({(void*)d, vec.size() * sizeof(T)});
    return true;
  };
  DevMesh& M = mesh_;
  M.C = (int)C; M.E = (int)E; M.N = (int)N; M.I = I;
  bool ok = true;
  const int *p_cnode, *p_cnbr, *p_cedge, *p_cinst, *p_eown, *p_enb, *p_esl, *p_esr, *p_einst, *p_icb;
  const unsigned char* p_cown;
  const double *p_bc, *p_fw, *p_area, *p_zn, *p_ze, *p_cek, *p_cnxc, *p_cnyc, *p_dry, *p_combo, *p_pw1, *p_enx, *p_eny,
      *p_etx, *p_ety, *p_ezm, *p_elmin, *p_nz, *p_cfl, *p_cor;
  const Pw2Rec* p_pw2;
  const SlotRec* p_srec;
  const int2* p_cslot;
  const EdgeRec* p_erec;
  const int4* p_eidx;
  ok = ok && up(img.cnode, p_cnode) && up(img.cnbr, p_cnbr) && up(img.cedge, p_cedge) && up(img.cinst, p_cinst);
  ok = ok && up(img.cown, p_cown) && up(img.bc, p_bc) && up(img.fwthr, p_fw) && up(img.area, p_area);
  ok = ok && up(img.zn, p_zn) && up(img.ze, p_ze) && up(img.cek, p_cek) && up(img.cnxc, p_cnxc) && up(img.cnyc, p_cnyc);
  ok = ok && up(img.dry, p_dry) && up(img.combo, p_combo) && up(img.pw1, p_pw1) && up(img.pw2, p_pw2);
  ok = ok && up(img.eown, p_eown) && up(img.enb, p_enb) && up(img.eslotl, p_esl) && up(img.eslotr, p_esr);
  ok = ok && up(img.einst, p_einst) && up(img.enx, p_enx) && up(img.eny, p_eny) && up(img.etx, p_etx);
  ok = ok && up(img.ety, p_ety) && up(img.ezm, p_ezm) && up(img.elmin, p_elmin) && up(img.nz, p_nz);
  ok = ok && up(img.inst_cell_begin, p_icb) && up(img.inst_cfl, p_cfl) && up(img.inst_cor, p_cor);
  ok = ok && up(img.srec, p_srec) && up(img.cslot, p_cslot) && up(img.erec, p_erec) && up(img.eidx, p_eidx);
  const int *p_nptr, *p_ncell;
  ok = ok && up(img.nptr, p_nptr) && up(img.ncell, p_ncell);
  if (!ok) {
    *st = 6;
    return std::string("device allocation or upload failed: ") + cudaGetErrorString(cudaGetLastError());
  }
  M.cnode = p_cnode; M.cnbr = p_cnbr; M.cedge = p_cedge; M.cinst = p_cinst; M.cown = p_cown;
  M.bc = p_bc; M.fwthr = p_fw; M.area = p_area; M.zn = p_zn; M.ze = p_ze; M.cek = p_cek;
  M.cnxc = p_cnxc; M.cnyc = p_cnyc; M.dry = p_dry; M.combo = p_combo; M.pw1 = p_pw1; M.pw2 = p_pw2;
  M.eown = p_eown; M.enb = p_enb; M.eslotl = p_esl; M.eslotr = p_esr; M.einst = p_einst;
  M.enx = p_enx; M.eny = p_eny; M.etx = p_etx; M.ety = p_ety; M.ezm = p_ezm; M.elmin = p_elmin;
  M.nz = p_nz; M.inst_cell_begin = p_icb; M.inst_cfl = p_cfl; M.inst_cor = p_cor;
  M.srec = p_srec; M.cslot = p_cslot; M.erec = p_erec; M.eidx = p_eidx;
  M.nptr = p_nptr; M.ncell = p_ncell;

  DevWork& Wk = work_;
  Wk.ew = dalloc<double>(3 * C); Wk.eu = dalloc<double>(3 * C); Wk.ev = dalloc<double>(3 * C);
  Wk.sx = dalloc<double>(3 * C); Wk.sy = dalloc<double>(3 * C);
  Wk.f0 = dalloc<double>(E); Wk.f1 = dalloc<double>(E); Wk.f2 = dalloc<double>(E);
  Wk.drain = dalloc<double>(C);
  Wk.maxwp = dalloc<unsigned long long>(N);
  Wk.pwlist = dalloc<int>(C);
  Wk.pwcount = dalloc<int>(1);
  Wk.pwrec = dalloc<double>(C);
  Wk.cls = dalloc<unsigned char>(C);
  Wk.ftape = nullptr;
  Wk.r = dalloc<unsigned long long>(I);
  Wk.dt = dalloc<double>(I);
  Wk.tsum = dalloc<double>(I);
  d_fixed_dt = dalloc<double>(I);  // per instance
  Wk.fixed_dt = d_fixed_dt;
  Wk.err = dalloc<unsigned>(1);
  M.err = Wk.err;
  for (int q = 0; q < 6; ++q) state_[q] = dalloc<double>(C);
  d_io = dalloc<double>(3 * C);
  d_ioflag = dalloc<unsigned>(1);
  if (!Wk.ew || !Wk.eu || !Wk.ev || !Wk.sx || !Wk.sy || !Wk.f0 || !Wk.f1 || !Wk.f2 || !Wk.drain || !Wk.maxwp ||
      !Wk.pwlist || !Wk.pwcount || !Wk.pwrec || !Wk.cls || !Wk.r || !Wk.dt || !Wk.tsum || !d_fixed_dt || !Wk.err ||
      !state_[5] || !d_io || !d_ioflag) {
    *st = 6;
    return "device allocation failed";
  }
  if (cudaMallocHost(&h_fixed_dt, sizeof(double)) != cudaSuccess) {
    *st = 6;
    return "pinned allocation failed";
  }
  cudaMemset(Wk.ew, 0, 3 * C * sizeof(double));
  cudaMemset(Wk.eu, 0, 3 * C * sizeof(double));
  cudaMemset(Wk.ev, 0, 3 * C * sizeof(double));
  cudaMemset(Wk.sx, 0, 3 * C * sizeof(double));
  cudaMemset(Wk.sy, 0, 3 * C * sizeof(double));
  cudaMemset(Wk.f0, 0, E * sizeof(double));
  cudaMemset(Wk.f1, 0, E * sizeof(double));
  cudaMemset(Wk.f2, 0, E * sizeof(double));
  cudaMemset(Wk.pwcount, 0, sizeof(int));
  cudaMemset(Wk.pwlist, 0, C * sizeof(int));  // every entry a valid cell id from the start
  cudaMemset(Wk.dt, 0, I * sizeof(double));
  cudaMemset(Wk.tsum, 0, I * sizeof(double));
  cudaMemset(Wk.err, 0, sizeof(unsigned));
  std::vector<unsigned long long> one(I, order_key(1.0));
  cudaMemcpy(Wk.r, one.data(), I * sizeof(unsigned long long), cudaMemcpyHostToDevice);
  if (cudaStreamCreateWithFlags(&own_stream_, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ev_fork_, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ev_join_, cudaEventDisableTiming) != cudaSuccess) {
    *st = 5;
    return "stream creation failed";
  }
  stream_ = own_stream_;
  k_init_nodes<<<nblocks(N, 256), 256, 0, stream_>>>(M, Wk);
  ++launches_;
  cudaError_t ce = cudaStreamSynchronize(stream_);
  if (ce != cudaSuccess) {
    *st = 5;
    return std::string("CUDA error during set-up: ") + cudaGetErrorString(ce);
  }
  host = std::move(inst);
  return "";
}

cudaError_t Engine::reset_pass() {
  k_init_nodes<<<nblocks(std::max(mesh_.N, 1), 256), 256, 0, stream_>>>(mesh_, work_);
  launches_ += 1;
  return cudaGetLastError();
}

void Engine::launch_recon1(const double* W, const double* U, const double* V, int latch_mode) {
  const int b = blk_[0], g = nblocks(mesh_.C, b);
  if (batched_) {
    if (cor0_) k_recon1<true, true><<<g, b, 0, stream_>>>(mesh_, work_, W, U, V, latch_mode);
    else k_recon1<true, false><<<g, b, 0, stream_>>>(mesh_, work_, W, U, V, latch_mode);
  } else {
    if (cor0_) k_recon1<false, true><<<g, b, 0, stream_>>>(mesh_, work_, W, U, V, latch_mode);
    else k_recon1<false, false><<<g, b, 0, stream_>>>(mesh_, work_, W, U, V, latch_mode);
  }
  ++launches_;
}

void Engine::launch_recon2(const double* W, const double* U, const double* V, cudaStream_t s) {
  const int b = blk_[0], g = std::max(1, std::min(nblocks(mesh_.C, b), 152 * 2048 / b));
  if (batched_) {
    if (cor0_) k_recon2<true, true><<<g, b, 0, s>>>(mesh_, work_, W, U, V);
    else k_recon2<true, false><<<g, b, 0, s>>>(mesh_, work_, W, U, V);
  } else {
    if (cor0_) k_recon2<false, true><<<g, b, 0, s>>>(mesh_, work_, W, U, V);
    else k_recon2<false, false><<<g, b, 0, s>>>(mesh_, work_, W, U, V);
  }
  ++launches_;
}

cudaError_t Engine::interface_values(const double* W, const double* U, const double* V, int latch_mode) {
  launch_recon1(W, U, V, latch_mode);
  launch_recon2(W, U, V, stream_);
  k_node_max_all<<<nblocks(std::max(mesh_.N, 1), 256), 256, 0, stream_>>>(mesh_, work_, W);
  ++launches_;
  return cudaGetLastError();
}

template <class FLUX, bool TAPE>
static void launch_flux_t(bool batched, int mode, int blocks, int b, cudaStream_t s, const DevMesh& m,
                          const DevWork& w, const double* W) {
  if (batched) {
    if (mode) k_flux<FLUX, true, 1, TAPE><<<blocks, b, 0, s>>>(m, w, W);
    else k_flux<FLUX, true, 0, TAPE><<<blocks, b, 0, s>>>(m, w, W);
  } else {
    if (mode) k_flux<FLUX, false, 1, TAPE><<<blocks, b, 0, s>>>(m, w, W);
    else k_flux<FLUX, false, 0, TAPE><<<blocks, b, 0, s>>>(m, w, W);
  }
}
template <class FLUX>
static void launch_flux(bool batched, int mode, int blocks, int b, cudaStream_t s, const DevMesh& m,
                        const DevWork& w, const double* W) {
  if (w.ftape) launch_flux_t<FLUX, true>(batched, mode, blocks, b, s, m, w, W);
  else launch_flux_t<FLUX, false>(batched, mode, blocks, b, s, m, w, W);
}
template <class FLUX>
static void launch_flux_pw(bool batched, int blocks, cudaStream_t s, const DevMesh& m, const DevWork& w,
                           const double* W) {
  if (w.ftape) {
    if (batched) k_flux_pw<FLUX, true, true><<<blocks, 128, 0, s>>>(m, w, W);
    else k_flux_pw<FLUX, false, true><<<blocks, 128, 0, s>>>(m, w, W);
  } else {
    if (batched) k_flux_pw<FLUX, true, false><<<blocks, 128, 0, s>>>(m, w, W);
    else k_flux_pw<FLUX, false, false><<<blocks, 128, 0, s>>>(m, w, W);
  }
}

cudaError_t Engine::fluxes(const double* W) { return fluxes(W, 0); }

cudaError_t Engine::fluxes(const double* W, int mode) {
  const int b = blk_[1], g = nblocks(mesh_.E, b);
  switch (flux_ * 3 + ws_) {
    case 0: launch_flux<HLL<Rusanov>>(batched_, mode, g, b, stream_, mesh_, work_, W); break;
    case 1: launch_flux<HLL<Davis>>(batched_, mode, g, b, stream_, mesh_, work_, W); break;
    case 2: launch_flux<HLL<Einfeldt>>(batched_, mode, g, b, stream_, mesh_, work_, W); break;
    case 3: launch_flux<HLLC<Rusanov>>(batched_, mode, g, b, stream_, mesh_, work_, W); break;
    case 4: launch_flux<HLLC<Davis>>(batched_, mode, g, b, stream_, mesh_, work_, W); break;
    default: launch_flux<HLLC<Einfeldt>>(batched_, mode, g, b, stream_, mesh_, work_, W); break;
  }
  launches_ += 1;
  return cudaGetLastError();
}

void Engine::fluxes_pw(const double* W, cudaStream_t s) {
  const int g = std::max(1, std::min((3 * (int)mesh_.C + 127) / 128, 152 * 8));
  switch (flux_ * 3 + ws_) {
    case 0: launch_flux_pw<HLL<Rusanov>>(batched_, g, s, mesh_, work_, W); break;
    case 1: launch_flux_pw<HLL<Davis>>(batched_, g, s, mesh_, work_, W); break;
    case 2: launch_flux_pw<HLL<Einfeldt>>(batched_, g, s, mesh_, work_, W); break;
    case 3: launch_flux_pw<HLLC<Rusanov>>(batched_, g, s, mesh_, work_, W); break;
    case 4: launch_flux_pw<HLLC<Davis>>(batched_, g, s, mesh_, work_, W); break;
    default: launch_flux_pw<HLLC<Einfeldt>>(batched_, g, s, mesh_, work_, W); break;
  }
  launches_ += 1;
}

cudaError_t Engine::launch_stage(const Stage& st, const double* const* in, const double* const* u0,
                                 double* const* out, bool first_stage_of_step, int latch_mode, cudaEvent_t* ev) {
  const int b = blk_[2];
  const int lm = first_stage_of_step ? latch_mode : 0;
  if (ev) cudaEventRecord(ev[0], stream_);
  launch_recon1(in[0], in[1], in[2], lm);
  if (ev) {
    // per-kernel timing: the kernels one after another
    cudaEventRecord(ev[1], stream_);
    launch_recon2(in[0], in[1], in[2], stream_);
    cudaEventRecord(ev[2], stream_);
    cudaError_t e = fluxes(in[0], 0);
    if (e != cudaSuccess) return e;
    cudaEventRecord(ev[3], stream_);
  } else {
    // PartWet2 and the fluxes next to partially-wet cells on the side stream,
    // beside the other edges' fluxes
    cudaEventRecord(ev_fork_, stream_);
    cudaStreamWaitEvent(side_, ev_fork_, 0);
    launch_recon2(in[0], in[1], in[2], side_);
    fluxes_pw(in[0], side_);
    cudaEventRecord(ev_join_, side_);
    cudaError_t e = fluxes(in[0], 1);
    if (e != cudaSuccess) return e;
    cudaStreamWaitEvent(stream_, ev_join_, 0);
  }
  k_drain<<<nblocks(mesh_.C, b), b, 0, stream_>>>(mesh_, work_, in[0]);
  if (ev) cudaEventRecord(ev[4], stream_);
  ++launches_;
  launch_update(st, in, u0, out, nullptr);
  if (ev) cudaEventRecord(ev[5], stream_);
  return cudaGetLastError();
}

template <bool BATCH, bool STORE_N, bool HALF>
static void update_kernel(int g, int b, cudaStream_t s, const DevMesh& m, const DevWork& w, const Stage& st,
                          const double* const* in, const double* const* u0, double* const* out, double* nst) {
  k_update<BATCH, STORE_N, HALF><<<g, b, 0, s>>>(m, w, in[0], in[1], in[2], u0[0], u0[1], u0[2], out[0], out[1],
                                                 out[2], st, nst);
}

void Engine::launch_update(const Stage& st, const double* const* in, const double* const* u0, double* const* out,
                           double* nst) {
  const int b = blk_[2], g = nblocks(mesh_.C, b);
  const bool half = !st.first && st.a == 0.5 && st.b == 0.5 && st.c == 0.5;
  const int sel = (batched_ ? 4 : 0) | (nst ? 2 : 0) | (half ? 1 : 0);
  switch (sel) {
    case 0: update_kernel<false, false, false>(g, b, stream_, mesh_, work_, st, in, u0, out, nst); break;
    case 1: update_kernel<false, false, true>(g, b, stream_, mesh_, work_, st, in, u0, out, nst); break;
    case 2: update_kernel<false, true, false>(g, b, stream_, mesh_, work_, st, in, u0, out, nst); break;
    case 3: update_kernel<false, true, true>(g, b, stream_, mesh_, work_, st, in, u0, out, nst); break;
    case 4: update_kernel<true, false, false>(g, b, stream_, mesh_, work_, st, in, u0, out, nst); break;
    case 5: update_kernel<true, false, true>(g, b, stream_, mesh_, work_, st, in, u0, out, nst); break;
    case 6: update_kernel<true, true, false>(g, b, stream_, mesh_, work_, st, in, u0, out, nst); break;
    default: update_kernel<true, true, true>(g, b, stream_, mesh_, work_, st, in, u0, out, nst); break;
  }
  ++launches_;
}

cudaError_t Engine::step_timed(int scheme, int latch_mode, double* acc) {
  const Scheme sc = scheme_of(scheme);
  double* S0[3] = {state(0, 0), state(0, 1), state(0, 2)};
  double* S1[3] = {state(1, 0), state(1, 1), state(1, 2)};
  cudaEvent_t ev[kMaxStages][6];
  for (auto& row : ev)
    for (auto& x : row) cudaEventCreate(&x);
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < sc.n && e == cudaSuccess; ++s) {
    const bool last = (s == sc.n - 1);
    const double* const* in = (s == 0) ? S0 : S1;
    double* const* out = last ? S0 : S1;
    e = launch_stage(sc.s[s], in, S0, out, s == 0, latch_mode, ev[s]);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  if (e == cudaSuccess) {
    for (int s = 0; s < sc.n; ++s)
      for (int k = 0; k < 5; ++k) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[s][k], ev[s][k + 1]);
        acc[k] += ms;
      }
    float tot = 0.f;
    cudaEventElapsedTime(&tot, ev[0][0], ev[sc.n - 1][5]);
    acc[5] += tot;
  }
  for (auto& row : ev)
    for (auto& x : row) cudaEventDestroy(x);
  return e;
}

void Engine::set_custom_scheme(const Scheme& sc) {
  custom_ = sc;
  for (auto& g : graphs_[kCustomScheme])
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

void Engine::set_blocks(const int blocks[3]) {
  bool same = true;
  for (int q = 0; q < 3; ++q) same = same && blk_[q] == blocks[q];
  if (same) return;
  for (int q = 0; q < 3; ++q) blk_[q] = blocks[q];
  for (auto& row : graphs_)
    for (auto& g : row)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
}

namespace {
std::mutex g_tune_mu;
std::map<std::array<int, 7>, std::array<int, 3>> g_tune_cache;
}  // namespace

cudaError_t Engine::snapshot(double* buf, bool restore) {
  const int64_t C = mesh_.C;
  cudaError_t r = cudaSuccess;
  for (int c = 0; c < 3 && r == cudaSuccess; ++c)
    r = restore ? cudaMemcpyAsync(state(0, c), buf + c * C, C * sizeof(double), cudaMemcpyDeviceToDevice, stream_)
                : cudaMemcpyAsync(buf + c * C, state(0, c), C * sizeof(double), cudaMemcpyDeviceToDevice, stream_);
  if (restore) {
    if (r == cudaSuccess) r = cudaMemsetAsync(work_.tsum, 0, mesh_.I * sizeof(double), stream_);
    if (r == cudaSuccess) r = cudaMemsetAsync(work_.dt, 0, mesh_.I * sizeof(double), stream_);
    if (r == cudaSuccess) r = cudaMemsetAsync(work_.err, 0, sizeof(unsigned), stream_);
  }
  return r;
}

cudaError_t Engine::autotune_blocks(int scheme) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int lg = 0;
  while ((1ll << (lg + 1)) <= (int64_t)mesh_.C) ++lg;
  const std::array<int, 7> key = {dev, flux_, ws_, batched_ ? 1 : 0, cor0_ ? 1 : 0, scheme, lg};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      set_blocks(it->second.data());
      return cudaSuccess;
    }
  }
  double* save = nullptr;
  e = cudaMalloc(&save, 3 * (size_t)mesh_.C * sizeof(double));
  if (e != cudaSuccess) return e;
  static const int kCand[3] = {64, 128, 256};
  const double inf = std::numeric_limits<double>::infinity();
  double t[3][3] = {{inf, inf, inf}, {inf, inf, inf}, {inf, inf, inf}};  // [group][candidate]
  e = snapshot(save, false);
  for (int ci = 0; ci < 3 && e == cudaSuccess; ++ci) {
    const int b3[3] = {kCand[ci], kCand[ci], kCand[ci]};
    set_blocks(b3);
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // rep 0 warms up
      double acc[6] = {0., 0., 0., 0., 0., 0.};
      e = snapshot(save, true);
      if (e == cudaSuccess) e = step_timed(scheme, 1, acc);
      if (e != cudaSuccess || rep == 0) continue;
      t[0][ci] = std::min(t[0][ci], acc[0] + acc[1]);
      t[1][ci] = std::min(t[1][ci], acc[2]);
      t[2][ci] = std::min(t[2][ci], acc[3] + acc[4]);
    }
  }
  int best[3] = {256, 256, 256};
  if (e == cudaSuccess)
    for (int g = 0; g < 3; ++g) {
      int k = 2;  // ties keep the largest block
      for (int ci = 1; ci >= 0; --ci)
        if (t[g][ci] < t[g][k]) k = ci;
      best[g] = kCand[k];
    }
  set_blocks(best);
  // back to the state before tuning
  cudaError_t e2 = snapshot(save, true);
  if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(stream_);
  cudaFree(save);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = {best[0], best[1], best[2]};
  }
  return e;
}

cudaError_t Engine::time_steps(int scheme, int n, float* ms) {
  double* save = nullptr;
  cudaError_t e = cudaMalloc(&save, 3 * (size_t)mesh_.C * sizeof(double));
  if (e != cudaSuccess) return e;
  cudaEvent_t a = nullptr, b = nullptr;
  e = snapshot(save, false);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e == cudaSuccess) e = run_graph(scheme, 1, 1);
  if (e == cudaSuccess) e = cudaEventRecord(a, stream_);
  if (e == cudaSuccess) e = run_graph(scheme, 1, n);
  if (e == cudaSuccess) e = cudaEventRecord(b, stream_);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  if (e == cudaSuccess) {
    e = cudaEventElapsedTime(ms, a, b);
    *ms /= (float)n;
  }
  cudaError_t e2 = snapshot(save, true);
  if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(stream_);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  cudaFree(save);
  return e == cudaSuccess ? e2 : e;
}

std::string Engine::set_layouts(std::vector<Layout>&& lay) {
  layouts = std::move(lay);
  bool any = false;
  for (const Layout& L : layouts) any = any || !L.identity();
  if (!any) return "";
  std::vector<int> from((size_t)mesh_.C);
  for (size_t q = 0; q < layouts.size(); ++q) {
    const int64_t c0 = cell_off[q], n = cell_off[q + 1] - c0;
    for (int64_t j = 0; j < n; ++j) from[c0 + j] = layouts[q].identity() ? (int)j : (int)layouts[q].cell_from[j];
  }
  std::vector<int> to((size_t)mesh_.C);
  for (size_t q = 0; q < layouts.size(); ++q) {
    const int64_t c0 = cell_off[q], n = cell_off[q + 1] - c0;
    for (int64_t j = 0; j < n; ++j) to[c0 + from[c0 + j]] = (int)(c0 + j);
  }
  d_cell_from = dalloc<int>(from.size());
  d_cell_to = dalloc<int>(to.size());
  if (!d_cell_from || !d_cell_to) return "device allocation failed";
  if (cudaMemcpy(d_cell_from, from.data(), from.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d_cell_to, to.data(), to.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return std::string("uploading the cell layout: ") + cudaGetErrorString(cudaGetLastError());
  return "";
}

std::string Engine::set_bathymetry(const std::vector<const double*>& z) {
  if (z.size() != host.size()) return "one bathymetry pointer per instance is required";
  for (size_t q = 0; q < host.size(); ++q) {
    if (!z[q]) continue;
    const HostInstance& h = host[q];
    const Layout* L = q < layouts.size() ? &layouts[q] : nullptr;
    for (int64_t p = 0; p < h.N; ++p)
      if (!std::isfinite(z[q][(L && !L->identity()) ? L->node_from[p] : p])) return "bathymetry has a non-finite value";
  }
  for (size_t q = 0; q < host.size(); ++q) {
    if (!z[q]) continue;
    HostInstance& h = host[q];
    const Layout* L = q < layouts.size() ? &layouts[q] : nullptr;
    for (int64_t p = 0; p < h.N; ++p) h.geom[3 * p + 2] = z[q][(L && !L->identity()) ? L->node_from[p] : p];
  }
  const int I = (int)host.size();
  HostImage img;
  img.resize(mesh_.C, mesh_.E, mesh_.N, I);
  for (int q = 0; q < I; ++q) precompute_instance(host[q], q, cell_off[q], edge_off[q], node_off[q], img);
  // the same arrays, in the order init uploaded them
  size_t k = 0;
  bool ok = true;
  auto refill = [&](auto& vec) {
    using T = typename std::remove_reference<decltype(vec)>::type::value_type;
    if (!ok || k >= mesh_arrays_.size() || mesh_arrays_[k].second != vec.size() * sizeof(T)) {
      ok = false;
      return;
    }
    ok = cudaMemcpyAsync(mesh_arrays_[k].first, vec.data(), vec.size() * sizeof(T), cudaMemcpyHostToDevice,
                         stream_) == cudaSuccess;
    ++k;
  };
  refill(img.cnode); refill(img.cnbr); refill(img.cedge); refill(img.cinst);
  refill(img.cown); refill(img.bc); refill(img.fwthr); refill(img.area);
  refill(img.zn); refill(img.ze); refill(img.cek); refill(img.cnxc); refill(img.cnyc);
  refill(img.dry); refill(img.combo); refill(img.pw1); refill(img.pw2);
  refill(img.eown); refill(img.enb); refill(img.eslotl); refill(img.eslotr);
  refill(img.einst); refill(img.enx); refill(img.eny); refill(img.etx);
  refill(img.ety); refill(img.ezm); refill(img.elmin); refill(img.nz);
  refill(img.inst_cell_begin); refill(img.inst_cfl); refill(img.inst_cor);
  refill(img.srec); refill(img.cslot); refill(img.erec); refill(img.eidx);
  refill(img.nptr); refill(img.ncell);
  if (!ok || k != mesh_arrays_.size()) return "re-uploading the mesh records failed";
  // the host image must outlive the asynchronous copies
  cudaError_t e = cudaStreamSynchronize(stream_);
  // the adjoint's tape and tables belong to the old bed
  if (adj_) {
    adjoint_state_delete(adj_);
    adj_ = nullptr;
  }
  return e == cudaSuccess ? "" : std::string("re-uploading the mesh records: ") + cudaGetErrorString(e);
}

cudaError_t Engine::update_only(const Stage& st, const double* const* in, const double* const* u0,
                                double* const* out, double* nst) {
  launch_update(st, in, u0, out, nst);
  return cudaGetLastError();
}

cudaError_t Engine::step(int scheme, int latch_mode) {
  const Scheme sc = scheme_of(scheme);
  double* S0[3] = {state(0, 0), state(0, 1), state(0, 2)};
  double* S1[3] = {state(1, 0), state(1, 1), state(1, 2)};
  for (int s = 0; s < sc.n; ++s) {
    const bool last = (s == sc.n - 1);
    const double* const* in = (s == 0) ? S0 : S1;
    double* const* out = last ? S0 : S1;
    cudaError_t e = launch_stage(sc.s[s], in, S0, out, s == 0, latch_mode);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t Engine::run_graph(int scheme, int latch_mode, int64_t n) {
  if (n <= 0) return cudaSuccess;
  cudaGraphExec_t& ge = graphs_[scheme][latch_mode];
  const int64_t per_step = launches_;
  if (!ge) {
    // capture on a private stream so that any caller stream (even the legacy
    // default one) can replay the graph
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return cudaGetLastError();
    cudaStream_t saved = stream_;
    stream_ = cap;
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
      stream_ = saved;
      cudaStreamDestroy(cap);
      return e;
    }
    e = step(scheme, latch_mode);
    cudaError_t e2 = cudaStreamEndCapture(cap, &g);
    stream_ = saved;
    cudaStreamDestroy(cap);
    if (e != cudaSuccess) return e;
    if (e2 != cudaSuccess) return e2;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      ge = nullptr;
      return e;
    }
    launches_ = per_step;  // capture launched nothing
  }
  const int64_t kernels_per_step = 6 * scheme_of(scheme).n;
  for (int64_t s = 0; s < n; ++s) {
    cudaError_t e = cudaGraphLaunch(ge, stream_);
    if (e != cudaSuccess) return e;
  }
  launches_ += kernels_per_step * n;
  return cudaSuccess;
}

}  // namespace swe
