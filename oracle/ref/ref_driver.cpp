// ref_driver.cpp -- C entry points over the reference's own solver classes.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/ref/build_ref.py together
// with the reference's unmodified src/*.cpp (two of them patched for Q1 and
// Q20, see that recipe) into oracle/_ref/libswe_ref.so; tests/ load it to pin
// the C restatement (oracle/swe_oracle.c) and to write golden vectors.
//
// Everything numerical below is the reference's code: Topology, Domain,
// VolumeField, SpaceDisc, TimeDisc, Fluxes::HLL/HLLC<Wavespeeds::*> and
// Solvers::Euler/SSPRK2/SSPRK3 (include/*.h, src/*.cpp).  The driver only
// builds them from flat arrays, runs them, and reads their fields back.
//
// Two loop orders:
//   literal -- the reference's own Solvers::X(td, dt), with its in-place
//              cell updates (src/Solvers.cpp:5-59) and its in-place pass 2 of
//              SpaceDisc::ComputeInterfaceValues (src/SpaceDisc.cpp:47-51);
//   jacobi  -- a time-scheme plugin (the reference's extension point,
//              include/Solvers.h:6-8) that runs the same reference calls but
//              evaluates every TimeDisc::RHS of a stage before writing any
//              cell, and takes every pass-2 reconstruction
//              (ReconstructPartWetCell2) before any pass-2 write.  This is the
//              order the GPU implements.
#include <Fluxes.h>
#include <Solvers.h>

#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace {

// raw read/write access to a value field's storage (BaseValueField::m_str is
// protected; the member pointer is formed inside a derived class)
struct FieldAccess : BaseValueField {
  static Storage<3>& raw(BaseValueField& f) { return f.*(&FieldAccess::m_str); }
  static const Storage<3>& raw(const BaseValueField& f) { return f.*(&FieldAccess::m_str); }
};

struct RefSpaceDisc : SpaceDisc {
  using SpaceDisc::SpaceDisc;

  Storage<1> max_wp_pass1;

  // SpaceDisc::ComputeInterfaceValues (src/SpaceDisc.cpp:33-52) with pass 2
  // reading the pass-1 node maxima only: every PartWet2 reconstruction is
  // taken before any of them writes.
  void ComputeInterfaceValuesJacobi() {
    m_max_wp = m_b.GetGeometry().row(2);
    const auto& m = m_b.GetTopology();
    for (size_t i = 0; i < (size_t)m.NumTriangles(); ++i) {
      if (IsDryCell(i)) {
        UpdateInterfaceValues(ReconstructDryCell(i));
      } else if (!IsFullWetCell(i)) {
        UpdateInterfaceValues(ReconstructPartWetCell1(i));
      } else {
        UpdateInterfaceValues(ReconstructFullWetCell(i));
      }
    }
    max_wp_pass1 = m_max_wp;
    std::vector<MUSCL> pass2;
    for (size_t i = 0; i < (size_t)m.NumTriangles(); ++i)
      if (IsPartWetCell(i)) pass2.push_back(ReconstructPartWetCell2(i));
    for (const auto& mu : pass2) UpdateInterfaceValues(mu);
  }

  const Storage<1>& MaxWp() const { return m_max_wp; }
};

enum { ORDER_JACOBI = 0, ORDER_LITERAL = 1 };

struct RefCase {
  PointArray geom;
  EdgeTagArray edge_nodes, edge_cells;
  TriangTagArray cell_nodes, cell_edges, cell_nbrs;
  std::unique_ptr<Eigen::Ref<PointArray>> gref;
  std::unique_ptr<Topology> topo;
  std::unique_ptr<Domain> dom;
  std::unique_ptr<RefSpaceDisc> sd;
  std::unique_ptr<TimeDisc> td;
  int order = ORDER_JACOBI;
  std::string error;
};

SpaceDisc::Fluxer fluxer(int flux, int ws) {
  switch (flux * 3 + ws) {
    case 0: return Fluxes::HLL<Wavespeeds::Rusanov>;
    case 1: return Fluxes::HLL<Wavespeeds::Davis>;
    case 2: return Fluxes::HLL<Wavespeeds::Einfeldt>;
    case 3: return Fluxes::HLLC<Wavespeeds::Rusanov>;
    case 4: return Fluxes::HLLC<Wavespeeds::Davis>;
    default: return Fluxes::HLLC<Wavespeeds::Einfeldt>;
  }
}

template <class A>
void fill_rows(A& a, Idx rows, const int64_t* src) {
  a.resize(rows, Eigen::NoChange);
  if (rows) std::memcpy(a.data(), src, sizeof(int64_t) * (size_t)(rows * a.cols()));
}

// ---------------------------------------------------------- jacobi schemes
// Each is Solvers::X (src/Solvers.cpp:5-59) with the stage's RHS evaluated for
// every cell before any cell is written; the update expressions are the
// reference's, operation for operation.
void interface_and_fluxes(RefSpaceDisc* sd) {
  sd->ComputeInterfaceValuesJacobi();
  sd->ComputeFluxes();
}

std::vector<Array<3>> all_rhs(TimeDisc* td, Idx n, double dt) {
  std::vector<Array<3>> r;
  r.reserve((size_t)n);
  for (Idx i = 0; i < n; ++i) r.push_back(td->RHS(i, dt));
  return r;
}

void JacobiEuler(RefSpaceDisc* sd, TimeDisc* td, double dt) {
  const Idx n = sd->GetDomain().GetTopology().NumTriangles();
  interface_and_fluxes(sd);
  const auto R = all_rhs(td, n, dt);
  for (Idx i = 0; i < n; ++i) sd->GetVolField().cons(i) += R[(size_t)i];
}

void JacobiSSPRK2(RefSpaceDisc* sd, TimeDisc* td, double dt) {
  const Idx n = sd->GetDomain().GetTopology().NumTriangles();
  interface_and_fluxes(sd);
  const VolumeField U0 = sd->GetVolField();
  auto R = all_rhs(td, n, dt);
  for (Idx i = 0; i < n; ++i) sd->GetVolField().cons(i) = U0.cons(i) + R[(size_t)i];

  interface_and_fluxes(sd);
  const VolumeField& U1 = sd->GetVolField();
  R = all_rhs(td, n, 0.5 * dt);
  for (Idx i = 0; i < n; ++i) sd->GetVolField().cons(i) = 0.5 * U0.cons(i) + 0.5 * U1.cons(i) + R[(size_t)i];
}

void JacobiSSPRK3(RefSpaceDisc* sd, TimeDisc* td, double dt) {
  const Idx n = sd->GetDomain().GetTopology().NumTriangles();
  interface_and_fluxes(sd);
  const VolumeField U0 = sd->GetVolField();
  auto R = all_rhs(td, n, dt);
  for (Idx i = 0; i < n; ++i) sd->GetVolField().cons(i) = U0.cons(i) + R[(size_t)i];

  interface_and_fluxes(sd);
  const VolumeField U1 = sd->GetVolField();
  R = all_rhs(td, n, 0.25 * dt);
  for (Idx i = 0; i < n; ++i) sd->GetVolField().cons(i) = 0.75 * U0.cons(i) + 0.25 * U1.cons(i) + R[(size_t)i];

  interface_and_fluxes(sd);
  const VolumeField& U2 = sd->GetVolField();
  R = all_rhs(td, n, (2. / 3.) * dt);
  for (Idx i = 0; i < n; ++i)
    sd->GetVolField().cons(i) = (1. / 3.) * U0.cons(i) + (2. / 3.) * U2.cons(i) + R[(size_t)i];
}

}  // namespace

extern "C" {

// mesh arrays as the reference holds them: geometry 3 x N column-major
// (x, y, z per node), int64 row-major E x 2 / E x 2 / C x 3 / C x 3 / C x 3;
// prim0 3 x C column-major (w, u, v per cell), stored as given.
void* swe_ref_create(int64_t num_nodes, int64_t num_edges, int64_t num_cells, const double* geom,
                     const int64_t* edge_nodes, const int64_t* edge_cells, const int64_t* cell_nodes,
                     const int64_t* cell_edges, const int64_t* cell_nbrs, const double* prim0, int flux, int ws,
                     double cor, int order) {
  auto c = std::make_unique<RefCase>();
  try {
    c->geom.resize(3, num_nodes);
    std::memcpy(c->geom.data(), geom, sizeof(double) * 3 * (size_t)num_nodes);
    fill_rows(c->edge_nodes, num_edges, edge_nodes);
    fill_rows(c->edge_cells, num_edges, edge_cells);
    fill_rows(c->cell_nodes, num_cells, cell_nodes);
    fill_rows(c->cell_edges, num_cells, cell_edges);
    fill_rows(c->cell_nbrs, num_cells, cell_nbrs);
    c->gref = std::make_unique<Eigen::Ref<PointArray>>(c->geom);
    c->topo = std::make_unique<Topology>(num_nodes, c->edge_nodes, c->edge_cells, c->cell_nodes, c->cell_edges,
                                         c->cell_nbrs);
    c->dom = std::make_unique<Domain>(*c->gref, *c->topo);
    VolumeField v0(*c->dom, (size_t)num_cells);
    std::memcpy(FieldAccess::raw(v0).data(), prim0, sizeof(double) * 3 * (size_t)num_cells);
    c->sd = std::make_unique<RefSpaceDisc>(fluxer(flux, ws), *c->dom, v0, cor, 0.0);
    c->td = std::make_unique<TimeDisc>(c->sd.get());
    c->order = order;
  } catch (const std::exception& e) {
    return nullptr;
  }
  return c.release();
}

void swe_ref_destroy(void* h) { delete static_cast<RefCase*>(h); }

// 0 on success; 1 and a message (swe_ref_error) when the reference throws
int swe_ref_step(void* h, int scheme, double dt) {
  auto* c = static_cast<RefCase*>(h);
  try {
    if (c->order == ORDER_LITERAL) {
      if (scheme == 0) Solvers::Euler(c->td.get(), dt);
      else if (scheme == 1) Solvers::SSPRK2(c->td.get(), dt);
      else Solvers::SSPRK3(c->td.get(), dt);
    } else {
      if (scheme == 0) JacobiEuler(c->sd.get(), c->td.get(), dt);
      else if (scheme == 1) JacobiSSPRK2(c->sd.get(), c->td.get(), dt);
      else JacobiSSPRK3(c->sd.get(), c->td.get(), dt);
    }
  } catch (const std::exception& e) {
    c->error = e.what();
    return 1;
  }
  return 0;
}

// SpaceDisc::ComputeInterfaceValues + ComputeFluxes in the case's order
int swe_ref_interface(void* h) {
  auto* c = static_cast<RefCase*>(h);
  try {
    if (c->order == ORDER_LITERAL) c->sd->ComputeInterfaceValues();
    else c->sd->ComputeInterfaceValuesJacobi();
    c->sd->ComputeFluxes();
  } catch (const std::exception& e) {
    c->error = e.what();
    return 1;
  }
  return 0;
}

const char* swe_ref_error(void* h) { return static_cast<RefCase*>(h)->error.c_str(); }

// SpaceDisc::GetMinLenToWavespeed (the ratio TimeDisc::CFLdt scales by 0.15)
double swe_ref_min_len_to_wavespeed(void* h) { return static_cast<RefCase*>(h)->sd->GetMinLenToWavespeed(); }
double swe_ref_cfl_dt(void* h) { return static_cast<RefCase*>(h)->td->CFLdt(); }

void swe_ref_get_prim(void* h, double* out) {
  auto* c = static_cast<RefCase*>(h);
  const auto& s = FieldAccess::raw(c->sd->GetVolField());
  std::memcpy(out, s.data(), sizeof(double) * 3 * (size_t)s.cols());
}

void swe_ref_set_prim(void* h, const double* in) {
  auto* c = static_cast<RefCase*>(h);
  auto& s = FieldAccess::raw(c->sd->GetVolField());
  std::memcpy(s.data(), in, sizeof(double) * 3 * (size_t)s.cols());
}

// interface values in the reference layout: edg / src 3 x 2E (slot 2e + (from < to)),
// fluxes 3 x E, node maxima N as pass 2 read them (jacobi: after pass 1;
// literal: the live array after pass 2)
void swe_ref_get_edge_fields(void* h, double* edg, double* src, double* f, double* max_wp) {
  auto* c = static_cast<RefCase*>(h);
  if (edg) {
    const auto& s = FieldAccess::raw(c->sd->GetEdgField());
    std::memcpy(edg, s.data(), sizeof(double) * 3 * (size_t)s.cols());
  }
  if (src) {
    const auto& s = FieldAccess::raw(c->sd->GetSrcField());
    std::memcpy(src, s.data(), sizeof(double) * 3 * (size_t)s.cols());
  }
  if (f) {
    const auto& s = c->sd->GetFluxes();
    std::memcpy(f, s.data(), sizeof(double) * 3 * (size_t)s.cols());
  }
  if (max_wp) {
    const auto& s = c->order == ORDER_LITERAL ? c->sd->MaxWp() : c->sd->max_wp_pass1;
    std::memcpy(max_wp, s.data(), sizeof(double) * (size_t)s.size());
  }
}

// 0 dry, 1 partially wet, 2 fully wet (MUSCLObject::Is*Cell, src/MUSCLObject.cpp:13-29)
void swe_ref_classify(void* h, int32_t* out) {
  auto* c = static_cast<RefCase*>(h);
  const Idx n = c->topo->NumTriangles();
  for (Idx i = 0; i < n; ++i) out[i] = c->sd->IsDryCell(i) ? 0 : (c->sd->IsFullWetCell(i) ? 2 : 1);
}

}  // extern "C"
