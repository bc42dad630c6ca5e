// Drives the GPU step through the reference's C++ API (swe_fvm_gb300.hpp),
// written the way the reference's own driver is (examples/Main.cpp): read a
// mesh and a state, fill a VolumeField through its prim(i) assigner, build
// SpaceDisc sd{fluxer, domain, v0}, run n SSPRK2 steps with dt = td.CFLdt(),
// write the state.
//
// usage: reference_api_main in.bin out.bin
//   in.bin : int64 N, E, C, n_steps; geometry 3N f64; edge_nodes 2E,
//            edge_cells 2E, cell_nodes 3C, cell_edges 3C, cell_neighbours 3C
//            int64; prim 3C f64
//   out.bin: the assigned initial field 3C f64, the final prim 3C f64, then
//            the sum of the dt used (f64)
// Exit codes: 0 ok, 2 DomainError, 3 SolverError, 4 I/O.
#include <cstdio>
#include <vector>

#include "swe_fvm_gb300.hpp"

template <class T>
static bool read(std::FILE* f, std::vector<T>& v, size_t n) {
  v.resize(n);
  return std::fread(v.data(), sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc != 3) return 4;
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 4;
  std::vector<int64_t> hdr, en, ec, cn, ce, ct;
  std::vector<double> geom, prim;
  bool ok = read(f, hdr, 4);
  const int64_t N = ok ? hdr[0] : 0, E = ok ? hdr[1] : 0, C = ok ? hdr[2] : 0, steps = ok ? hdr[3] : 0;
  ok = ok && read(f, geom, 3 * N) && read(f, en, 2 * E) && read(f, ec, 2 * E) && read(f, cn, 3 * C) &&
       read(f, ce, 3 * C) && read(f, ct, 3 * C) && read(f, prim, 3 * C);
  std::fclose(f);
  if (!ok) return 4;
  double t = 0.;
  std::vector<double> v0_out;
  try {
    Topology topo(N, E, C, en.data(), ec.data(), cn.data(), ce.data(), ct.data());
    Domain dom(geom.data(), topo);
    VolumeField v0{dom, (size_t)C};
    for (int64_t i = 0; i < C; ++i) v0.prim(i) = {prim[3 * i], prim[3 * i + 1], prim[3 * i + 2]};
    v0_out.assign(v0.data(), v0.data() + 3 * C);
    SpaceDisc sd{Fluxes::HLLC<Wavespeeds::Einfeldt>, dom, v0};
    TimeDisc td(&sd);
    for (int64_t n = 0; n < steps; ++n) {
      const double dt = td.CFLdt();
      Solvers::SSPRK2(&td, dt);
      t += dt;
    }
    sd.GetVolField(prim.data());
  } catch (const DomainError& e) {
    std::fprintf(stderr, "DomainError: %s\n", e.what());
    return 2;
  } catch (const SolverError& e) {
    std::fprintf(stderr, "SolverError: %s\n", e.what());
    return 3;
  }
  std::FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 4;
  std::fwrite(v0_out.data(), sizeof(double), v0_out.size(), o);
  std::fwrite(prim.data(), sizeof(double), prim.size(), o);
  std::fwrite(&t, sizeof(double), 1, o);
  std::fclose(o);
  return 0;
}
