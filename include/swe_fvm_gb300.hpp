// swe_fvm_gb300.hpp -- the reference's C++ API over the C ABI (header only).
//
// Code written against the reference's SpaceDisc / TimeDisc / Solvers /
// Fluxes / Wavespeeds (include/SpaceDisc.h:20-48, include/TimeDisc.h:4-25,
// include/Solvers.h:4-10, include/Fluxes.h:14-111, src/Fluxes.cpp:5-26)
// compiles against this header with the GPU step underneath:
//
//   Topology topo(numNodes, numEdges, numCells, edgeNodes, edgeCells, cellNodes, cellEdges, cellNeighbours);
//   Domain dom(geometry, topo);
//   SpaceDisc sd(Fluxes::HLLC<Wavespeeds::Einfeldt>, dom, v0);
//   TimeDisc td(&sd);
//   Solvers::SSPRK2(&td, td.CFLdt());
//
// Differences, all at the edges of the API: arrays are plain pointers in the
// reference's layouts (geometry 3 x N column-major, int64 row-major topology,
// the 3 x C primitive field) instead of Eigen storage; SpaceDisc copies
// them to the device; field getters copy into caller buffers.  Status codes
// of the C ABI come back as the reference's exceptions (include/Exceptions.h:
// 4-10): DomainError for meshes and arguments, SolverError for the step.
// Link with -lswe_gb300 -lcudart.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "swe_fvm_gb300.h"

struct DomainError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct SolverError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

namespace swe_gpu_detail {
inline void check_create(swe_status st) {
  if (st == SWE_OK) return;
  const std::string msg = swe_last_error(nullptr);
  if (st == SWE_ERR_INVALID_MESH || st == SWE_ERR_INVALID_ARGUMENT) throw DomainError(msg);
  throw SolverError(msg);
}
inline void check(swe_ctx* ctx, swe_status st) {
  if (st == SWE_OK) return;
  const std::string msg = ctx ? swe_last_error(ctx) : "invalid context";
  if (st == SWE_ERR_INVALID_ARGUMENT) throw DomainError(msg);
  throw SolverError(msg);
}
}  // namespace swe_gpu_detail

// Wave-speed plugins (src/Fluxes.cpp:5-26): selectors of the device functors.
namespace Wavespeeds {
struct Kind {
  int32_t id;
};
inline constexpr Kind Rusanov{SWE_WS_RUSANOV};
inline constexpr Kind Davis{SWE_WS_DAVIS};
inline constexpr Kind Einfeldt{SWE_WS_EINFELDT};
}  // namespace Wavespeeds

// Flux plugins (include/Fluxes.h:14-111): Fluxes::HLL<W> and Fluxes::HLLC<W>
// name the compiled device flux for wave speed W, as the reference's function
// templates name its host fluxes.
namespace Fluxes {
struct Fluxer {
  int32_t flux;
  int32_t wavespeed;
};
template <const Wavespeeds::Kind& W>
inline constexpr Fluxer HLL{SWE_FLUX_HLL, W.id};
template <const Wavespeeds::Kind& W>
inline constexpr Fluxer HLLC{SWE_FLUX_HLLC, W.id};
}  // namespace Fluxes

// Topology (include/TriangMesh.h:14-65): a view of the caller's arrays, like
// the reference's (which holds references).
struct Topology {
  Topology(int64_t numNodes, int64_t numEdges, int64_t numCells, const int64_t* edgeNodes, const int64_t* edgeCells,
           const int64_t* cellNodes, const int64_t* cellEdges, const int64_t* cellNeighbours)
      : num_nodes(numNodes), num_edges(numEdges), num_cells(numCells), edge_nodes(edgeNodes),
        edge_cells(edgeCells), cell_nodes(cellNodes), cell_edges(cellEdges), cell_neighbours(cellNeighbours) {}
  int64_t NumNodes() const noexcept { return num_nodes; }
  int64_t NumEdges() const noexcept { return num_edges; }
  int64_t NumTriangles() const noexcept { return num_cells; }
  bool IsEdgeBoundary(int64_t e) const noexcept { return edge_cells[2 * e + 1] < 0; }  // src/TriangMesh.cpp:5-7

  int64_t num_nodes, num_edges, num_cells;
  const int64_t *edge_nodes, *edge_cells, *cell_nodes, *cell_edges, *cell_neighbours;
};

// Domain (include/Bathymetry.h:12-49): the node geometry (x, y, z per node).
struct Domain {
  Domain(const double* geometry, const Topology& topo) : geometry(geometry), topo(topo) {}
  const Topology& GetTopology() const noexcept { return topo; }
  const double* geometry;
  const Topology& topo;
};

// VolumeField (include/ValueField.h:31-78 with VolumeIndexer and
// VolumeDomainWrapper): the 3 x C primitive field (w, u, v per cell) of a
// domain, with the cell bathymetry b(i) the centroid z (src/ValueField.cpp:
// 8-10).  prim(i) = {w, u, v} writes through PrimAssigner's rules and
// cons(i) = {h, hu, hv} through ConsAssigner's (src/Assigners.cpp:8-44),
// including their dry clamps and thin-film desingularisation; += / -= read the
// current value back the same way.  Intermediate products are held in
// volatile doubles so that a compiler contracting multiply-adds cannot change
// the reference's rounding.
class VolumeField {
 public:
  using Value = std::array<double, 3>;

  explicit VolumeField(const Domain& b, size_t size = 0) : b_(&b), str_(3 * size, 0.) {}
  size_t Size() const noexcept { return str_.size() / 3; }
  void Resize(size_t size) { str_.resize(3 * size, 0.); }
  const double* data() const noexcept { return str_.data(); }
  double* data() noexcept { return str_.data(); }

  // centroid z: (P(tp) * (1/3, 1/3, 1/3)) row 2 (src/Bathymetry.cpp:24-27)
  double b(int64_t i) const {
    const Topology& t = b_->GetTopology();
    const double k = 1. / 3.;
    const int64_t* tp = t.cell_nodes + 3 * i;
    volatile double a0 = b_->geometry[3 * tp[0] + 2] * k, a1 = b_->geometry[3 * tp[1] + 2] * k;
    volatile double s = a0 + a1;
    volatile double a2 = b_->geometry[3 * tp[2] + 2] * k;
    return s + a2;
  }
  double w(int64_t i) const { return str_[3 * i]; }
  double u(int64_t i) const { return str_[3 * i + 1]; }
  double v(int64_t i) const { return str_[3 * i + 2]; }
  double h(int64_t i) const { return w(i) - b(i); }
  double hu(int64_t i) const { return h(i) * u(i); }
  double hv(int64_t i) const { return h(i) * v(i); }
  Value prim(int64_t i) const { return {w(i), u(i), v(i)}; }
  Value cons(int64_t i) const { return {h(i), hu(i), hv(i)}; }

  // PrimAssigner (src/Assigners.cpp:8-20)
  struct PrimAssigner {
    VolumeField& f;
    int64_t i;
    void operator=(const Value& r) {
      const double bb = f.b(i);
      double* c = f.str_.data() + 3 * i;
      const double hh = r[0] - bb;
      if (!(hh > 1e-12)) {
        c[0] = bb; c[1] = 0.; c[2] = 0.;
        return;
      }
      c[0] = r[0]; c[1] = r[1]; c[2] = r[2];
      if (hh < 1e-3) {
        volatile double h2 = hh * hh;
        volatile double num = std::sqrt(2.) * hh;
        const double sc = num / std::sqrt(h2 + 1e-6);
        c[1] *= sc;
        c[2] *= sc;
      }
    }
    Value Get() const { return static_cast<const VolumeField&>(f).prim(i); }
    void operator+=(const Value& r) { *this = Value{Get()[0] + r[0], Get()[1] + r[1], Get()[2] + r[2]}; }
    void operator-=(const Value& r) { *this = Value{Get()[0] - r[0], Get()[1] - r[1], Get()[2] - r[2]}; }
  };
  // ConsAssigner (src/Assigners.cpp:22-44)
  struct ConsAssigner {
    VolumeField& f;
    int64_t i;
    void operator=(const Value& r) {
      const double bb = f.b(i);
      double* c = f.str_.data() + 3 * i;
      const double hh = r[0];
      if (!(hh > 1e-12)) {
        c[0] = bb; c[1] = 0.; c[2] = 0.;
        return;
      }
      double ih;
      if (hh < 1e-3) {
        volatile double h2 = hh * hh;
        volatile double h3 = h2 * hh;
        volatile double h4 = h3 * hh;
        volatile double num = std::sqrt(2.) * hh;
        ih = num / std::sqrt(h4 + 1e-12);
      } else {
        ih = 1. / hh;
      }
      c[0] = hh + bb;
      c[1] = r[1] * ih;
      c[2] = r[2] * ih;
    }
    Value Get() const {  // (w - b, u (w - b), v (w - b))
      const double hh = f.w(i) - f.b(i);
      return {hh, f.u(i) * hh, f.v(i) * hh};
    }
    void operator+=(const Value& r) {
      const Value g = Get();
      *this = Value{g[0] + r[0], g[1] + r[1], g[2] + r[2]};
    }
    void operator-=(const Value& r) {
      const Value g = Get();
      *this = Value{g[0] - r[0], g[1] - r[1], g[2] - r[2]};
    }
  };
  PrimAssigner prim(int64_t i) { return PrimAssigner{*this, i}; }
  ConsAssigner cons(int64_t i) { return ConsAssigner{*this, i}; }

 private:
  const Domain* b_;
  std::vector<double> str_;
};

// SpaceDisc (include/SpaceDisc.h:20-48) on the GPU.  `options` carries the
// settings the reference does not have (CFL coefficient, device order, block
// size); its defaults are swe_params_default's.
class SpaceDisc {
 public:
  SpaceDisc(const Fluxes::Fluxer& fluxer, const Domain& b, const double* v0, double cor = 0, double tau = 0,
            const swe_params* options = nullptr)
      : cor_(cor), tau_(tau) {
    swe_params p;
    if (options) p = *options;
    else swe_params_default(&p);
    p.flux = fluxer.flux;
    p.wavespeed = fluxer.wavespeed;
    p.cor = cor;
    p.tau = tau;
    const Topology& t = b.GetTopology();
    const swe_mesh m{t.num_nodes,  t.num_edges,      t.num_cells,      b.geometry,        t.edge_nodes,
                     t.edge_cells, t.cell_nodes,     t.cell_edges,     t.cell_neighbours};
    swe_gpu_detail::check_create(swe_create(&m, v0, &p, &ctx_));
    num_cells_ = t.num_cells;
    num_edges_ = t.num_edges;
    num_nodes_ = t.num_nodes;
    cfl_ = p.cfl;
  }
  // the reference's construction: SpaceDisc sd{fluxer, domain, v0, cor, tau}
  // copies v0 (src/MUSCLObject.cpp:8-11)
  SpaceDisc(const Fluxes::Fluxer& fluxer, const Domain& b, const VolumeField& v0, double cor = 0, double tau = 0,
            const swe_params* options = nullptr)
      : SpaceDisc(fluxer, b, v0.data(), cor, tau, options) {}
  SpaceDisc(const SpaceDisc&) = delete;
  SpaceDisc& operator=(const SpaceDisc&) = delete;
  SpaceDisc(SpaceDisc&& o) noexcept { *this = std::move(o); }
  SpaceDisc& operator=(SpaceDisc&& o) noexcept {
    std::swap(ctx_, o.ctx_);
    cor_ = o.cor_;
    tau_ = o.tau_;
    cfl_ = o.cfl_;
    num_cells_ = o.num_cells_;
    num_edges_ = o.num_edges_;
    num_nodes_ = o.num_nodes_;
    return *this;
  }
  ~SpaceDisc() {
    if (ctx_) swe_destroy(ctx_);
  }

  void ComputeInterfaceValues() { swe_gpu_detail::check(ctx_, swe_compute_interface_values(ctx_)); }
  void ComputeFluxes() { swe_gpu_detail::check(ctx_, swe_compute_fluxes(ctx_)); }
  double GetMinLenToWavespeed() const {
    double r = 0.;
    swe_gpu_detail::check(ctx_, swe_min_len_to_wavespeed(ctx_, &r));
    return r;
  }
  double GetCor() const noexcept { return cor_; }
  double GetTau() const noexcept { return tau_; }

  // the 3 x C primitive field (w, u, v per cell), the caller's cell order
  void GetVolField(double* out) const { swe_gpu_detail::check(ctx_, swe_get_prim(ctx_, out)); }
  std::vector<double> GetVolField() const {
    std::vector<double> v(3 * (size_t)num_cells_);
    GetVolField(v.data());
    return v;
  }
  void SetVolField(const double* in) { swe_gpu_detail::check(ctx_, swe_set_prim(ctx_, in)); }
  // edge fields in the reference's 3 x 2E EdgeIndexer order, fluxes 3 x E
  std::vector<double> GetEdgField() const { return edge_values(true); }
  std::vector<double> GetSrcField() const { return edge_values(false); }
  std::vector<double> GetFluxes() const {
    std::vector<double> f(3 * (size_t)num_edges_);
    swe_gpu_detail::check(ctx_, swe_get_fluxes(ctx_, f.data()));
    return f;
  }

  double cfl() const noexcept { return cfl_; }
  swe_ctx* handle() const noexcept { return ctx_; }

 private:
  std::vector<double> edge_values(bool edg) const {
    std::vector<double> v(6 * (size_t)num_edges_);
    swe_gpu_detail::check(ctx_, swe_get_edge_values(ctx_, edg ? v.data() : nullptr, edg ? nullptr : v.data()));
    return v;
  }
  swe_ctx* ctx_ = nullptr;
  double cor_ = 0., tau_ = 0., cfl_ = 0.15;
  int64_t num_cells_ = 0, num_edges_ = 0, num_nodes_ = 0;
};

// TimeDisc (include/TimeDisc.h:4-25).
class TimeDisc {
 public:
  explicit TimeDisc(SpaceDisc* sd = nullptr) : sd_(sd) {}
  SpaceDisc* GetSpaceDisc() noexcept { return sd_; }
  const SpaceDisc* GetSpaceDisc() const noexcept { return sd_; }
  void SetSpaceDisc(SpaceDisc* sd) noexcept { sd_ = sd; }
  // the CFL coefficient (0.15 in the reference) times the last flux pass's ratio
  double CFLdt() const { return sd_->cfl() * sd_->GetMinLenToWavespeed(); }

 private:
  SpaceDisc* sd_;
};

// Solvers (include/Solvers.h:4-10): one step with a given dt.  Custom runs
// the table defined by swe_set_scheme.
namespace Solvers {
inline void step(TimeDisc* const td, int32_t scheme, double dt) {
  swe_ctx* c = td->GetSpaceDisc()->handle();
  swe_gpu_detail::check(c, swe_step(c, scheme, dt));
}
inline void Euler(TimeDisc* const td, double dt) { step(td, SWE_SCHEME_EULER, dt); }
inline void SSPRK2(TimeDisc* const td, double dt) { step(td, SWE_SCHEME_SSPRK2, dt); }
inline void SSPRK3(TimeDisc* const td, double dt) { step(td, SWE_SCHEME_SSPRK3, dt); }
inline void Custom(TimeDisc* const td, double dt) { step(td, SWE_SCHEME_CUSTOM, dt); }
}  // namespace Solvers
