// swe_abi.cu -- the extern "C" boundary declared in include/swe_fvm_gb300.h.
//
// A swe_ctx is an Engine over one instance; a swe_batch is an Engine over many.
// Every entry point validates its arguments, catches C++ exceptions and turns
// CUDA errors into status codes with a message (the reference throws
// DomainError / SolverError / std::runtime_error, include/Exceptions.h:4-10).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/swe_fvm_gb300.h"
#include "swe_engine.cuh"
#include "swe_layout.cuh"

using swe::Engine;
using swe::HostInstance;

struct swe_ctx {
  Engine eng;
  std::string err;
  int flux = 1, ws = 2;
  double cfl = 0.15;
  bool primed = false;
};

struct swe_batch {
  Engine eng;
  std::string err;
  bool primed = false;
};

namespace {

thread_local std::string g_create_error;

// NVTX range over an entry point (host side: for graph replays it spans the
// enqueue), named after the entry point, for timeline tools; free when no tool
// is attached.
struct Trace {
  explicit Trace(const char* name) { nvtxRangePushA(name); }
  ~Trace() { nvtxRangePop(); }
  Trace(const Trace&) = delete;
  Trace& operator=(const Trace&) = delete;
};

swe_status fail(std::string* slot, swe_status st, const std::string& msg) {
  if (slot) *slot = msg;
  else g_create_error = msg;
  return st;
}

swe_status cuda_fail(std::string* slot, cudaError_t e, const char* where) {
  return fail(slot, SWE_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Interleave / de-interleave between the reference's 3 x C column-major
// primitive field (the caller's cell order) and the engine's three component
// arrays (device order; from[i] = the caller's row of device cell i, or null
// when the two orders agree).
__global__ void k_pack(const double* __restrict__ W, const double* __restrict__ U, const double* __restrict__ V,
                       double* __restrict__ out, int n, const int* __restrict__ from) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int r = from ? from[i] : i;
    out[3 * r] = W[i];
    out[3 * r + 1] = U[i];
    out[3 * r + 2] = V[i];
  }
}
__global__ void k_unpack(const double* __restrict__ in, double* __restrict__ W, double* __restrict__ U,
                         double* __restrict__ V, int n, unsigned* bad, const int* __restrict__ from) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int r = from ? from[i] : i;
    const double w = in[3 * r], u = in[3 * r + 1], v = in[3 * r + 2];
    W[i] = w;
    U[i] = u;
    V[i] = v;
    if (bad && !(isfinite(w) && isfinite(u) && isfinite(v))) atomicOr(bad, 1u);
  }
}

swe_status read_instance(const swe_mesh* m, const swe_params* p, HostInstance* h, std::string* why) {
  if (!m || !m->geometry || !m->edge_nodes || !m->edge_cells || !m->cell_nodes || !m->cell_edges ||
      !m->cell_neighbours) {
    *why = "mesh or one of its arrays is NULL";
    return SWE_ERR_INVALID_ARGUMENT;
  }
  if (m->num_nodes <= 0 || m->num_edges <= 0 || m->num_cells <= 0) {
    *why = "mesh sizes must be positive";
    return SWE_ERR_INVALID_MESH;
  }
  if (!(p->cfl > 0.) || !std::isfinite(p->cfl) || !std::isfinite(p->cor)) {
    *why = "cfl must be positive and finite, cor finite";
    return SWE_ERR_INVALID_ARGUMENT;
  }
  h->C = m->num_cells;
  h->E = m->num_edges;
  h->N = m->num_nodes;
  h->geom.assign(m->geometry, m->geometry + 3 * m->num_nodes);
  h->en.assign(m->edge_nodes, m->edge_nodes + 2 * m->num_edges);
  h->ec.assign(m->edge_cells, m->edge_cells + 2 * m->num_edges);
  h->cn.assign(m->cell_nodes, m->cell_nodes + 3 * m->num_cells);
  h->ce.assign(m->cell_edges, m->cell_edges + 3 * m->num_cells);
  h->ct.assign(m->cell_neighbours, m->cell_neighbours + 3 * m->num_cells);
  h->cfl = p->cfl;
  h->cor = p->cor;
  return SWE_OK;
}

// Validates one instance in the caller's numbering (so that messages name the
// caller's indices), then picks its device layout and rewrites it in that
// order.
swe_status lay_out(HostInstance* h, int strategy, swe::Layout* L, std::string* why) {
  std::string err = swe::validate_instance(*h);
  if (!err.empty()) {
    *why = err;
    return SWE_ERR_INVALID_MESH;
  }
  if (strategy == swe::kLayoutKeep) {
    *L = swe::Layout{};
    return SWE_OK;
  }
  HostInstance o;
  *L = swe::choose_layout(*h, strategy, nullptr, &o);
  if (!L->identity()) *h = std::move(o);
  return SWE_OK;
}

// Device position of the caller's (global) cell index.
int64_t device_cell(const Engine& g, int64_t c) {
  const size_t q = std::upper_bound(g.cell_off.begin(), g.cell_off.end(), c) - g.cell_off.begin() - 1;
  const int64_t c0 = g.cell_off[q];
  const swe::Layout& L = g.layouts[q];
  return L.identity() ? c : c0 + L.cell_to[c - c0];
}

// Device-ordered rows (w values per cell or node, instances concatenated) to
// the caller's order.
void cells_to_caller(const Engine& g, const double* dev, double* out, int w) {
  for (size_t q = 0; q < g.layouts.size(); ++q) {
    const int64_t c0 = g.cell_off[q], n = g.cell_off[q + 1] - c0;
    const swe::Layout& L = g.layouts[q];
    for (int64_t j = 0; j < n; ++j) {
      const int64_t d = c0 + (L.identity() ? j : L.cell_from[j]);
      for (int c = 0; c < w; ++c) out[w * d + c] = dev[w * (c0 + j) + c];
    }
  }
}
void nodes_to_caller(const Engine& g, const double* dev, double* out) {
  for (size_t q = 0; q < g.layouts.size(); ++q) {
    const int64_t n0 = g.node_off[q], n = g.node_off[q + 1] - n0;
    const swe::Layout& L = g.layouts[q];
    for (int64_t j = 0; j < n; ++j) out[n0 + (L.identity() ? j : L.node_from[j])] = dev[n0 + j];
  }
}
bool reordered(const Engine& g) { return g.d_cell_from != nullptr; }

// Engine::adjoint_backward with its per-cell and per-node gradients returned
// in the caller's order.
std::string adjoint_backward_caller(Engine& g, const double* trace_grads, double* grad_prim0, double* grad_z) {
  if (!reordered(g)) return g.adjoint_backward(trace_grads, grad_prim0, grad_z);
  std::vector<double> gp(3 * (size_t)g.C()), gz((size_t)g.N());
  std::string e = g.adjoint_backward(trace_grads, gp.data(), gz.data());
  if (!e.empty()) return e;
  cells_to_caller(g, gp.data(), grad_prim0, 3);
  nodes_to_caller(g, gz.data(), grad_z);
  return "";
}

// Times the block sizes (swe_params.block == 0) and re-primes the flux pass.
swe_status tune(Engine& eng, std::string* err);

constexpr const char* kSchemeMsg = "scheme must be 0, 1, 2 or SWE_SCHEME_CUSTOM once defined";

// A caller's Shu-Osher table (swe_set_scheme) as engine stages; "" or why not.
std::string make_scheme(int32_t n, const double* a, const double* b, const double* c, swe::Scheme* out) {
  if (n < 1 || n > swe::kMaxStages) return "n_stages must be 1 to " + std::to_string(swe::kMaxStages);
  if (!a || !b || !c) return "a, b and c are required";
  swe::Scheme sc{};
  sc.n = n;
  for (int s = 0; s < n; ++s) {
    if (!std::isfinite(a[s]) || !std::isfinite(b[s]) || !(c[s] > 0.) || !std::isfinite(c[s]))
      return "stage " + std::to_string(s) + ": a and b must be finite and c positive and finite";
    if (std::fabs(a[s] + b[s] - 1.) > 1e-14)
      return "stage " + std::to_string(s) + ": a + b must be 1 (a consistent combination of states)";
    // stage 0 reads the step's initial state: U0 + RHS(dt) when it is plainly
    // that, else the general combination (both terms then read U0)
    const bool first = s == 0 && c[s] == 1. && ((a[s] == 1. && b[s] == 0.) || (a[s] == 0. && b[s] == 1.));
    sc.s[s] = swe::Stage{first, first ? 0. : a[s], first ? 0. : b[s], first ? 1. : c[s]};
  }
  *out = sc;
  return "";
}

// Meshes from this many cells up choose their device order (SWE_REORDER_AUTO)
// by timing each candidate; smaller ones by the gather cost model.
constexpr int64_t kTimedLayoutCells = 1 << 16;
constexpr int kTimedLayoutSteps = 10;

swe_status check_params(const swe_params* p, std::string* why) {
  if (p->flux < 0 || p->flux > 1) {
    *why = "flux must be SWE_FLUX_HLL or SWE_FLUX_HLLC";
    return SWE_ERR_INVALID_ARGUMENT;
  }
  if (p->wavespeed < 0 || p->wavespeed > 2) {
    *why = "wavespeed must be SWE_WS_RUSANOV, SWE_WS_DAVIS or SWE_WS_EINFELDT";
    return SWE_ERR_INVALID_ARGUMENT;
  }
  if (p->reorder < SWE_REORDER_AUTO || p->reorder > SWE_REORDER_RCM) {
    *why = "reorder must be SWE_REORDER_AUTO, SWE_REORDER_KEEP, SWE_REORDER_MORTON or SWE_REORDER_RCM";
    return SWE_ERR_INVALID_ARGUMENT;
  }
  if (p->block != 0 && (p->block < 32 || p->block > 256 || p->block % 32 != 0)) {
    *why = "block must be 0 (tuned) or a multiple of 32 from 32 to 256";
    return SWE_ERR_INVALID_ARGUMENT;
  }
  return SWE_OK;
}

swe_status upload_prim(Engine& eng, const double* prim, int64_t c0, int64_t n, std::string* err) {
  // one copy of the interleaved field into the staging buffer, then a device
  // unpack that also flags non-finite values
  unsigned* flag = eng.d_ioflag;
  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(unsigned), eng.stream());
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(eng.d_io, prim, 3 * n * sizeof(double), cudaMemcpyHostToDevice, eng.stream());
  if (e == cudaSuccess) {
    k_unpack<<<(int)((n + 255) / 256), 256, 0, eng.stream()>>>(eng.d_io, eng.state(0, 0) + c0, eng.state(0, 1) + c0,
                                                                eng.state(0, 2) + c0, (int)n, flag,
                                                                eng.d_cell_from ? eng.d_cell_from + c0 : nullptr);
    e = cudaGetLastError();
  }
  unsigned h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(eng.stream());
  if (e != cudaSuccess) return cuda_fail(err, e, "uploading the state");
  if (h) return fail(err, SWE_ERR_NONFINITE, "state has a non-finite value");
  return SWE_OK;
}

swe_status download_prim(Engine& eng, double* prim, int64_t c0, int64_t n, std::string* err) {
  k_pack<<<(int)((n + 255) / 256), 256, 0, eng.stream()>>>(eng.state(0, 0) + c0, eng.state(0, 1) + c0,
                                                            eng.state(0, 2) + c0, eng.d_io, (int)n,
                                                            eng.d_cell_from ? eng.d_cell_from + c0 : nullptr);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(prim, eng.d_io, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(eng.stream());
  if (e != cudaSuccess) return cuda_fail(err, e, "downloading the state");
  return SWE_OK;
}

// Reads and clears nothing: reports the device error word.
swe_status check_device(Engine& eng, std::string* err) {
  cudaError_t e = cudaStreamSynchronize(eng.stream());
  if (e != cudaSuccess) return cuda_fail(err, e, "device execution");
  unsigned flags = 0;
  e = cudaMemcpy(&flags, eng.work().err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(err, e, "reading the device error word");
  if (flags & swe::kErrBadIndex)
    return fail(err, SWE_ERR_INVALID_MESH, "a kernel gathered an index out of range (checked build)");
  if (flags & swe::kErrNonFinite) return fail(err, SWE_ERR_NONFINITE, "a cell update produced a non-finite value");
  return SWE_OK;
}

// Priming flux pass so that CFLdt() is defined before the first step.
swe_status prime(Engine& eng, std::string* err) {
  cudaError_t e = eng.reset_pass();
  if (e == cudaSuccess) e = eng.interface_values(eng.state(0, 0), eng.state(0, 1), eng.state(0, 2), 0);
  if (e == cudaSuccess) e = eng.fluxes(eng.state(0, 0));
  if (e == cudaSuccess) e = eng.reset_pass();
  if (e != cudaSuccess) return cuda_fail(err, e, "priming flux pass");
  return SWE_OK;
}

swe_status tune(Engine& eng, std::string* err) {
  Trace trace("swe_tune_blocks");
  cudaError_t e = eng.autotune_blocks(1);
  if (e != cudaSuccess) return cuda_fail(err, e, "tuning the block sizes");
  return prime(eng, err);
}

// A context over one validated instance already in the device order of L.
swe_status build_ctx(HostInstance&& h, swe::Layout&& L, const swe_params& p, const double* prim0,
                     std::unique_ptr<swe_ctx>* out, std::string* why) {
  std::unique_ptr<swe_ctx> ctx(new swe_ctx());
  ctx->flux = p.flux;
  ctx->ws = p.wavespeed;
  ctx->cfl = p.cfl;
  int ist = 0;
  const int64_t C = h.C;
  std::vector<HostInstance> inst(1);
  inst[0] = std::move(h);
  std::string e = ctx->eng.init(std::move(inst), p.flux, p.wavespeed, p.block, &ist, false);
  if (!e.empty()) return fail(why, (swe_status)ist, e);
  std::vector<swe::Layout> lay(1);
  lay[0] = std::move(L);
  e = ctx->eng.set_layouts(std::move(lay));
  if (!e.empty()) return fail(why, SWE_ERR_CUDA, e);
  swe_status st = upload_prim(ctx->eng, prim0, 0, C, why);
  if (st == SWE_OK) st = prime(ctx->eng, why);
  if (st == SWE_OK && p.block == 0) st = tune(ctx->eng, why);
  if (st != SWE_OK) return st;
  // creation returns with the priming pass done (the caller may move the
  // context to another stream next)
  cudaError_t e2 = cudaStreamSynchronize(ctx->eng.stream());
  if (e2 != cudaSuccess) return cuda_fail(why, e2, "priming flux pass");
  *out = std::move(ctx);
  return SWE_OK;
}

// SWE_REORDER_AUTO on a large mesh or batch: builds the context (swe_ctx) or
// batch (swe_batch) in each order (the caller's, Morton, RCM; a batch takes one
// order for all its instances) through build(strategy, &candidate), times
// kTimedLayoutSteps graph-replayed SSPRK2 steps of each from the initial state
// (twice, keeping the faster), and keeps the fastest; another order replaces
// the current best only when it is more than 2 % faster.  At most two exist at
// once, and a candidate is skipped when the device has no room for it beside
// the best one.
template <class T, class Build>
swe_status choose_timed(Build&& build, std::unique_ptr<T>* out, std::string* why) {
  Trace trace("swe_time_layouts");
  static const int kCand[3] = {SWE_REORDER_KEEP, SWE_REORDER_MORTON, SWE_REORDER_RCM};
  std::unique_ptr<T> best;
  float best_ms = 0.f;
  for (int s : kCand) {
    if (best) {
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) break;
      if (free_b < best->eng.device_bytes() + best->eng.device_bytes() / 4 + (size_t(256) << 20)) break;
    }
    std::unique_ptr<T> c;
    swe_status st = build(s, &c);
    if (st != SWE_OK) {
      if (best) break;  // keep what already works
      return st;
    }
    float ms = 0.f, ms2 = 0.f;
    cudaError_t e = c->eng.time_steps(1, kTimedLayoutSteps, &ms);
    if (e == cudaSuccess) e = c->eng.time_steps(1, kTimedLayoutSteps, &ms2);
    if (e != cudaSuccess) return cuda_fail(why, e, "timing a device order");
    st = prime(c->eng, why);
    if (st == SWE_OK && cudaStreamSynchronize(c->eng.stream()) != cudaSuccess)
      st = cuda_fail(why, cudaGetLastError(), "priming flux pass");
    if (st != SWE_OK) return st;
    ms = std::min(ms, ms2);
    if (!best || ms < 0.98f * best_ms) {
      best = std::move(c);
      best_ms = ms;
    }
  }
  *out = std::move(best);
  return SWE_OK;
}

swe_status create_timed(const HostInstance& h, const swe_params& p, const double* prim0,
                        std::unique_ptr<swe_ctx>* out, std::string* why) {
  auto build = [&](int s, std::unique_ptr<swe_ctx>* c) {
    swe::Layout L = swe::make_layout(h, s);
    HostInstance d = L.identity() ? h : swe::apply_layout(h, L);
    return build_ctx(std::move(d), std::move(L), p, prim0, c, why);
  };
  return choose_timed<swe_ctx>(build, out, why);
}

// A batch over validated instances already in the device orders of lay.
swe_status build_batch(std::vector<HostInstance>&& inst, std::vector<swe::Layout>&& lay, const swe_params& p0,
                       const double* const* prim0, std::unique_ptr<swe_batch>* out, std::string* why) {
  const int n = (int)inst.size();
  std::unique_ptr<swe_batch> b(new swe_batch());
  int ist = 0;
  std::string e = b->eng.init(std::move(inst), p0.flux, p0.wavespeed, p0.block, &ist, true);
  if (!e.empty()) return fail(why, (swe_status)ist, e);
  e = b->eng.set_layouts(std::move(lay));
  if (!e.empty()) return fail(why, SWE_ERR_CUDA, e);
  for (int q = 0; q < n; ++q) {
    const int64_t c0 = b->eng.cell_off[q], c = b->eng.cell_off[q + 1] - c0;
    swe_status st = upload_prim(b->eng, prim0[q], c0, c, why);
    if (st != SWE_OK) {
      *why = "instance " + std::to_string(q) + ": " + *why;
      return st;
    }
  }
  swe_status st = prime(b->eng, why);
  if (st == SWE_OK && p0.block == 0) st = tune(b->eng, why);
  if (st != SWE_OK) return st;
  cudaError_t e2 = cudaStreamSynchronize(b->eng.stream());
  if (e2 != cudaSuccess) return cuda_fail(why, e2, "priming flux pass");
  *out = std::move(b);
  return SWE_OK;
}

// SWE_REORDER_AUTO for a batch of 65,536 cells or more: choose_timed over
// batches whose instances all take one order.
swe_status create_batch_timed(const std::vector<HostInstance>& inst, const swe_params& p0, const double* const* prim0,
                              std::unique_ptr<swe_batch>* out, std::string* why) {
  auto build = [&](int s, std::unique_ptr<swe_batch>* c) {
    const size_t n = inst.size();
    std::vector<HostInstance> d(n);
    std::vector<swe::Layout> L(n);
    for (size_t q = 0; q < n; ++q) {
      L[q] = swe::make_layout(inst[q], s);
      d[q] = L[q].identity() ? inst[q] : swe::apply_layout(inst[q], L[q]);
    }
    return build_batch(std::move(d), std::move(L), p0, prim0, c, why);
  };
  return choose_timed<swe_batch>(build, out, why);
}

#define SWE_GUARD_BEGIN try {
#define SWE_GUARD_END(slot)                                           \
  }                                                                   \
  catch (const std::bad_alloc&) {                                     \
    return fail(slot, SWE_ERR_OUT_OF_MEMORY, "host allocation failed"); \
  }                                                                   \
  catch (const std::exception& ex) {                                  \
    return fail(slot, SWE_ERR_INVALID_ARGUMENT, ex.what());           \
  }

}  // namespace

extern "C" {

swe_status swe_params_default(swe_params* p) {
  if (!p) return SWE_ERR_INVALID_ARGUMENT;
  p->flux = SWE_FLUX_HLLC;
  p->wavespeed = SWE_WS_EINFELDT;
  p->cor = 0.;
  p->tau = 0.;
  p->cfl = 0.15;
  p->reorder = SWE_REORDER_AUTO;
  p->block = 0;
  return SWE_OK;
}

swe_status swe_create(const swe_mesh* mesh, const double* prim0, const swe_params* params, swe_ctx** out) {
  Trace trace("swe_create");
  SWE_GUARD_BEGIN
  if (!out) return fail(nullptr, SWE_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (!prim0) return fail(nullptr, SWE_ERR_INVALID_ARGUMENT, "prim0 is NULL");
  swe_params p;
  if (params) p = *params;
  else swe_params_default(&p);
  std::string why;
  swe_status st = check_params(&p, &why);
  if (st != SWE_OK) return fail(nullptr, st, why);
  HostInstance h;
  st = read_instance(mesh, &p, &h, &why);
  if (st != SWE_OK) return fail(nullptr, st, why);
  std::unique_ptr<swe_ctx> ctx;
  if (p.reorder == SWE_REORDER_AUTO && h.C >= kTimedLayoutCells) {
    why = swe::validate_instance(h);
    if (!why.empty()) return fail(nullptr, SWE_ERR_INVALID_MESH, why);
    st = create_timed(h, p, prim0, &ctx, &why);
  } else {
    swe::Layout L;
    st = lay_out(&h, p.reorder, &L, &why);
    if (st == SWE_OK) st = build_ctx(std::move(h), std::move(L), p, prim0, &ctx, &why);
  }
  if (st != SWE_OK) return fail(nullptr, st, why);
  *out = ctx.release();
  return SWE_OK;
  SWE_GUARD_END(nullptr)
}

swe_status swe_destroy(swe_ctx* ctx) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  cudaStreamSynchronize(ctx->eng.stream());
  delete ctx;
  return SWE_OK;
}

swe_status swe_set_stream(swe_ctx* ctx, void* stream) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  ctx->eng.set_stream(stream ? (cudaStream_t)stream : nullptr);
  return SWE_OK;
}

swe_status swe_step(swe_ctx* ctx, int32_t scheme, double dt) {
  Trace trace("swe_step");
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  if (!ctx->eng.has_scheme(scheme)) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, kSchemeMsg);
  if (!(dt > 0.) || !std::isfinite(dt)) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
  cudaError_t e = cudaMemcpyAsync(ctx->eng.d_fixed_dt, &dt, sizeof(double), cudaMemcpyHostToDevice, ctx->eng.stream());
  // one replay of the step's CUDA graph (captured on first use)
  if (e == cudaSuccess) e = ctx->eng.run_graph(scheme, 2, 1);
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_step");
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_run(swe_ctx* ctx, int32_t scheme, double dt, int64_t n_steps) {
  Trace trace("swe_run");
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  if (!ctx->eng.has_scheme(scheme)) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, kSchemeMsg);
  if (!(dt > 0.) || !std::isfinite(dt)) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
  if (n_steps < 0) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "n_steps must be >= 0");
  cudaError_t e = cudaMemcpyAsync(ctx->eng.d_fixed_dt, &dt, sizeof(double), cudaMemcpyHostToDevice, ctx->eng.stream());
  if (e == cudaSuccess) e = ctx->eng.run_graph(scheme, 2, n_steps);
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_run");
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_run_cfl(swe_ctx* ctx, int32_t scheme, int64_t n_steps, double* t_elapsed) {
  Trace trace("swe_run_cfl");
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  if (!ctx->eng.has_scheme(scheme)) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, kSchemeMsg);
  if (n_steps < 0) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "n_steps must be >= 0");
  cudaError_t e = ctx->eng.run_graph(scheme, 1, n_steps);
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_run_cfl");
  if (t_elapsed) {
    e = cudaMemcpyAsync(t_elapsed, ctx->eng.work().tsum, sizeof(double), cudaMemcpyDeviceToHost, ctx->eng.stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->eng.stream());
    if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_run_cfl");
  }
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_min_len_to_wavespeed(swe_ctx* ctx, double* r) {
  if (!ctx || !r) return SWE_ERR_INVALID_ARGUMENT;
  unsigned long long k = 0;
  cudaError_t e = cudaMemcpyAsync(&k, ctx->eng.work().r, sizeof(k), cudaMemcpyDeviceToHost, ctx->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->eng.stream());
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_min_len_to_wavespeed");
  *r = swe::order_val(k);
  return SWE_OK;
}

swe_status swe_cfl_dt(swe_ctx* ctx, double* dt) {
  if (!ctx || !dt) return SWE_ERR_INVALID_ARGUMENT;
  double r = 0.;
  swe_status st = swe_min_len_to_wavespeed(ctx, &r);
  if (st != SWE_OK) return st;
  *dt = ctx->cfl * r;
  return SWE_OK;
}

swe_status swe_compute_interface_values(swe_ctx* ctx) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  Engine& g = ctx->eng;
  cudaError_t e = g.reset_pass();
  if (e == cudaSuccess) e = g.interface_values(g.state(0, 0), g.state(0, 1), g.state(0, 2), 0);
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_compute_interface_values");
  return SWE_OK;
}

swe_status swe_compute_fluxes(swe_ctx* ctx) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  cudaError_t e = ctx->eng.fluxes(ctx->eng.state(0, 0));
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_compute_fluxes");
  return SWE_OK;
}

swe_status swe_integrals(swe_ctx* ctx, double* out3) {
  Trace trace("swe_integrals");
  if (!ctx || !out3) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  cudaError_t e = ctx->eng.integrals(0, ctx->eng.C(), out3);
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_integrals");
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_get_prim(swe_ctx* ctx, double* prim_out) {
  Trace trace("swe_get_prim");
  if (!ctx || !prim_out) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return download_prim(ctx->eng, prim_out, 0, ctx->eng.C(), &ctx->err);
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_set_prim(swe_ctx* ctx, const double* prim_in) {
  Trace trace("swe_set_prim");
  if (!ctx || !prim_in) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  // like assigning the reference's volume field: CFLdt() keeps the ratio of
  // the last flux pass
  return upload_prim(ctx->eng, prim_in, 0, ctx->eng.C(), &ctx->err);
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_get_prim_device(swe_ctx* ctx, double* out) {
  if (!ctx || !out) return SWE_ERR_INVALID_ARGUMENT;
  Engine& g = ctx->eng;
  const int n = g.C();
  k_pack<<<(n + 255) / 256, 256, 0, g.stream()>>>(g.state(0, 0), g.state(0, 1), g.state(0, 2), out, n, g.d_cell_from);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_get_prim_device");
  return SWE_OK;
}

swe_status swe_set_prim_device(swe_ctx* ctx, const double* in) {
  if (!ctx || !in) return SWE_ERR_INVALID_ARGUMENT;
  Engine& g = ctx->eng;
  const int n = g.C();
  k_unpack<<<(n + 255) / 256, 256, 0, g.stream()>>>(in, g.state(0, 0), g.state(0, 1), g.state(0, 2), n, nullptr,
                                                     g.d_cell_from);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_set_prim_device");
  return SWE_OK;
}

swe_status swe_get_edge_values(swe_ctx* ctx, double* edg_out, double* src_out) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  Engine& g = ctx->eng;
  const int64_t C = g.C(), E = g.E();
  std::vector<double> ew(3 * C), eu(3 * C), ev(3 * C), sx(3 * C), sy(3 * C);
  const swe::DevWork& w = g.work();
  cudaError_t e = cudaStreamSynchronize(g.stream());
  if (e == cudaSuccess) e = cudaMemcpy(ew.data(), w.ew, 3 * C * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(eu.data(), w.eu, 3 * C * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(ev.data(), w.ev, 3 * C * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(sx.data(), w.sx, 3 * C * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(sy.data(), w.sy, 3 * C * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_get_edge_values");
  const HostInstance& h = g.host[0];
  const swe::Layout& L = g.layouts[0];
  if (edg_out) std::memset(edg_out, 0, 6 * E * sizeof(double));
  if (src_out) std::memset(src_out, 0, 6 * E * sizeof(double));
  for (int64_t i = 0; i < C; ++i)
    for (int k = 0; k < 3; ++k) {
      // the slot's edge, cell and neighbour in the caller's numbering
      int64_t ed = h.ce[3 * i + k], nb = h.ct[3 * i + k], ci = i;
      if (!L.identity()) {
        ed = L.edge_from[ed];
        nb = nb >= 0 ? L.cell_from[nb] : nb;
        ci = L.cell_from[i];
      }
      const int64_t id = 2 * ed + (ci < nb ? 1 : 0);  // EdgeIndexer::Id (include/ValueField.h:70-75)
      const int64_t s = k * C + i;
      if (edg_out) {
        edg_out[3 * id] = ew[s];
        edg_out[3 * id + 1] = eu[s];
        edg_out[3 * id + 2] = ev[s];
      }
      if (src_out) {
        src_out[3 * id + 1] = sx[s];
        src_out[3 * id + 2] = sy[s];
      }
    }
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_get_fluxes(swe_ctx* ctx, double* f_out) {
  if (!ctx || !f_out) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  Engine& g = ctx->eng;
  const int64_t E = g.E();
  std::vector<double> a(E), b(E), c(E);
  cudaError_t e = cudaStreamSynchronize(g.stream());
  if (e == cudaSuccess) e = cudaMemcpy(a.data(), g.work().f0, E * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(b.data(), g.work().f1, E * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(c.data(), g.work().f2, E * sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_get_fluxes");
  const swe::Layout& L = g.layouts[0];
  for (int64_t q = 0; q < E; ++q) {
    const int64_t d = L.identity() ? q : L.edge_from[q];
    f_out[3 * d] = a[q];
    f_out[3 * d + 1] = b[q];
    f_out[3 * d + 2] = c[q];
  }
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_get_node_max(swe_ctx* ctx, double* max_out) {
  if (!ctx || !max_out) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  Engine& g = ctx->eng;
  const int64_t N = g.N();
  std::vector<unsigned long long> k(N);
  cudaError_t e = cudaStreamSynchronize(g.stream());
  if (e == cudaSuccess) e = cudaMemcpy(k.data(), g.work().maxwp, N * sizeof(k[0]), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_get_node_max");
  std::vector<double> v(N);
  for (int64_t q = 0; q < N; ++q) v[q] = swe::order_val(k[q]);
  nodes_to_caller(g, v.data(), max_out);
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_time_kernels(swe_ctx* ctx, int32_t scheme, int64_t reps, double* out_ms) {
  if (!ctx || !out_ms) return SWE_ERR_INVALID_ARGUMENT;
  if (!ctx->eng.has_scheme(scheme) || reps <= 0) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "bad scheme or reps");
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t r = 0; r < reps; ++r) {
    cudaError_t e = ctx->eng.step_timed(scheme, 1, acc);
    if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_time_kernels");
  }
  const int n_st = ctx->eng.scheme_of(scheme).n;
  for (int k = 0; k < 5; ++k) out_ms[k] = acc[k] / (double)(reps * n_st);
  out_ms[5] = acc[5] / (double)reps;
  return SWE_OK;
}

swe_status swe_num_cells(swe_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return SWE_ERR_INVALID_ARGUMENT;
  *n = ctx->eng.C();
  return SWE_OK;
}

swe_status swe_launch_count(swe_ctx* ctx, int64_t* n) {
  if (!ctx || !n) return SWE_ERR_INVALID_ARGUMENT;
  *n = ctx->eng.launches();
  return SWE_OK;
}

swe_status swe_synchronize(swe_ctx* ctx) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  return check_device(ctx->eng, &ctx->err);
}

const char* swe_last_error(swe_ctx* ctx) {
  if (!ctx) return g_create_error.c_str();
  return ctx->err.c_str();
}

swe_status swe_adjoint_forward(swe_ctx* ctx, int32_t scheme, int64_t n_steps, int64_t checkpoint_every,
                               int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every, double* traces_out) {
  Trace trace("swe_adjoint_forward");
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  if (!ctx->eng.has_scheme(scheme) || n_steps <= 0 || checkpoint_every <= 0 || n_gauges < 0 || obs_every <= 0)
    return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "bad scheme, step counts or gauge count");
  if (n_gauges > 0 && (!gauge_cells || !traces_out))
    return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "gauge_cells and traces_out are required");
  std::vector<int> g(n_gauges);
  for (int q = 0; q < n_gauges; ++q) {
    if (gauge_cells[q] < 0 || gauge_cells[q] >= ctx->eng.C())
      return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "gauge cell out of range");
    g[q] = (int)device_cell(ctx->eng, gauge_cells[q]);
  }
  std::string e = ctx->eng.adjoint_forward(scheme, n_steps, checkpoint_every, g.data(), n_gauges, obs_every,
                                           traces_out);
  if (!e.empty()) return fail(&ctx->err, SWE_ERR_CUDA, e);
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_adjoint_backward(swe_ctx* ctx, const double* trace_grads, double* grad_prim0, double* grad_bathymetry) {
  Trace trace("swe_adjoint_backward");
  if (!ctx || !grad_prim0 || !grad_bathymetry) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  std::string e = adjoint_backward_caller(ctx->eng, trace_grads, grad_prim0, grad_bathymetry);
  if (!e.empty()) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, e);
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

// gauges in the caller's numbering -> device positions; "" or why not
std::string map_gauges(const Engine& g, int32_t n_gauges, const int64_t* gauge_cells, std::vector<int>* out) {
  out->assign(n_gauges > 0 ? n_gauges : 0, 0);
  for (int q = 0; q < n_gauges; ++q) {
    if (gauge_cells[q] < 0 || gauge_cells[q] >= g.C()) return "gauge cell out of range";
    (*out)[q] = (int)device_cell(g, gauge_cells[q]);
  }
  return "";
}

swe_status run_traces_common(Engine& eng, std::string* err, int32_t scheme, int64_t n_steps, const double* dts,
                             int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every, double* traces_out) {
  if (!eng.has_scheme(scheme) || n_steps <= 0 || n_gauges < 0 || obs_every <= 0 || !dts)
    return fail(err, SWE_ERR_INVALID_ARGUMENT, "bad scheme, step counts, gauge count or dts");
  if (n_gauges > 0 && (!gauge_cells || !traces_out))
    return fail(err, SWE_ERR_INVALID_ARGUMENT, "gauge_cells and traces_out are required");
  for (int64_t k = 0; k < n_steps * (int64_t)eng.I(); ++k)
    if (!(dts[k] > 0.) || !std::isfinite(dts[k]))
      return fail(err, SWE_ERR_INVALID_ARGUMENT, "every dt must be positive and finite");
  std::vector<int> g;
  std::string e = map_gauges(eng, n_gauges, gauge_cells, &g);
  if (!e.empty()) return fail(err, SWE_ERR_INVALID_ARGUMENT, e);
  e = eng.run_traces(scheme, n_steps, dts, g.data(), n_gauges, obs_every, traces_out);
  if (!e.empty()) return fail(err, SWE_ERR_CUDA, e);
  return SWE_OK;
}

swe_status adjoint_forward_device_common(Engine& eng, std::string* err, int32_t scheme, int64_t n_steps,
                                         int64_t checkpoint_every, int32_t n_gauges, const int64_t* gauge_cells,
                                         int64_t obs_every, double* traces_out) {
  if (!eng.has_scheme(scheme) || n_steps <= 0 || checkpoint_every <= 0 || n_gauges < 0 || obs_every <= 0)
    return fail(err, SWE_ERR_INVALID_ARGUMENT, "bad scheme, step counts or gauge count");
  if (n_gauges > 0 && (!gauge_cells || !traces_out))
    return fail(err, SWE_ERR_INVALID_ARGUMENT, "gauge_cells and traces_out are required");
  std::vector<int> g;
  std::string e = map_gauges(eng, n_gauges, gauge_cells, &g);
  if (!e.empty()) return fail(err, SWE_ERR_INVALID_ARGUMENT, e);
  e = eng.adjoint_forward(scheme, n_steps, checkpoint_every, g.data(), n_gauges, obs_every, traces_out, true);
  if (!e.empty()) return fail(err, SWE_ERR_CUDA, e);
  return SWE_OK;
}

swe_status set_bathymetry_common(Engine& eng, std::string* err, const std::vector<const double*>& z) {
  std::string e = eng.set_bathymetry(z);
  if (e.empty()) return SWE_OK;
  if (e.find("non-finite") != std::string::npos) return fail(err, SWE_ERR_NONFINITE, e);
  return fail(err, SWE_ERR_CUDA, e);
}

swe_status swe_run_traces(swe_ctx* ctx, int32_t scheme, int64_t n_steps, const double* dts, int32_t n_gauges,
                          const int64_t* gauge_cells, int64_t obs_every, double* traces_out) {
  Trace trace("swe_run_traces");
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return run_traces_common(ctx->eng, &ctx->err, scheme, n_steps, dts, n_gauges, gauge_cells, obs_every, traces_out);
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_set_bathymetry(swe_ctx* ctx, const double* z) {
  Trace trace("swe_set_bathymetry");
  if (!ctx || !z) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return set_bathymetry_common(ctx->eng, &ctx->err, std::vector<const double*>{z});
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_prime(swe_ctx* ctx) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return prime(ctx->eng, &ctx->err);
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_adjoint_forward_device(swe_ctx* ctx, int32_t scheme, int64_t n_steps, int64_t checkpoint_every,
                                      int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every,
                                      double* traces_out) {
  Trace trace("swe_adjoint_forward_device");
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return adjoint_forward_device_common(ctx->eng, &ctx->err, scheme, n_steps, checkpoint_every, n_gauges, gauge_cells,
                                       obs_every, traces_out);
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_adjoint_backward_device(swe_ctx* ctx, const double* trace_grads, double* grad_prim0,
                                       double* grad_bathymetry) {
  Trace trace("swe_adjoint_backward_device");
  if (!ctx || !grad_prim0 || !grad_bathymetry) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  std::string e = ctx->eng.adjoint_backward(trace_grads, grad_prim0, grad_bathymetry, true);
  if (!e.empty()) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, e);
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_adjoint_prepare(swe_ctx* ctx) {
  Trace trace("swe_adjoint_prepare");
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  std::string e = ctx->eng.adjoint_init();
  if (!e.empty()) return fail(&ctx->err, SWE_ERR_CUDA, e);
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_adjoint_set_regularisation(swe_ctx* ctx, double depth) {
  if (!ctx || !(depth >= 0.) || !std::isfinite(depth)) return SWE_ERR_INVALID_ARGUMENT;
  ctx->eng.set_adjoint_regularisation(depth);
  return SWE_OK;
}

swe_status swe_adjoint_dts(swe_ctx* ctx, double* dts_out) {
  if (!ctx || !dts_out) return SWE_ERR_INVALID_ARGUMENT;
  std::string e = ctx->eng.adjoint_dts(dts_out);
  if (!e.empty()) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, e);
  return SWE_OK;
}

swe_status swe_set_scheme(swe_ctx* ctx, int32_t n_stages, const double* a, const double* b, const double* c) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  swe::Scheme sc;
  std::string e = make_scheme(n_stages, a, b, c, &sc);
  if (!e.empty()) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, e);
  ctx->eng.set_custom_scheme(sc);
  return SWE_OK;
  SWE_GUARD_END(&ctx->err)
}

swe_status swe_get_time(swe_ctx* ctx, double* t) {
  if (!ctx || !t) return SWE_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaMemcpyAsync(t, ctx->eng.work().tsum, sizeof(double), cudaMemcpyDeviceToHost, ctx->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->eng.stream());
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_get_time");
  return SWE_OK;
}

swe_status swe_set_time(swe_ctx* ctx, double t) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  if (!std::isfinite(t)) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "t must be finite");
  cudaError_t e = cudaMemcpyAsync(ctx->eng.work().tsum, &t, sizeof(double), cudaMemcpyHostToDevice, ctx->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->eng.stream());
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_set_time");
  return SWE_OK;
}

swe_status swe_set_min_len_to_wavespeed(swe_ctx* ctx, double r) {
  if (!ctx) return SWE_ERR_INVALID_ARGUMENT;
  if (!(r > 0.) || !std::isfinite(r)) return fail(&ctx->err, SWE_ERR_INVALID_ARGUMENT, "r must be positive and finite");
  const unsigned long long k = swe::order_key(r);
  cudaError_t e = cudaMemcpyAsync(ctx->eng.work().r, &k, sizeof(k), cudaMemcpyHostToDevice, ctx->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->eng.stream());
  if (e != cudaSuccess) return cuda_fail(&ctx->err, e, "swe_set_min_len_to_wavespeed");
  return SWE_OK;
}

swe_status swe_get_tuning(swe_ctx* ctx, int32_t* out4) {
  if (!ctx || !out4) return SWE_ERR_INVALID_ARGUMENT;
  out4[0] = ctx->eng.layouts.empty() ? 0 : ctx->eng.layouts[0].strategy;
  for (int q = 0; q < 3; ++q) out4[1 + q] = ctx->eng.blocks()[q];
  return SWE_OK;
}

swe_status swe_layout_plan(const swe_mesh* mesh, int32_t strategy, int64_t* cell_from, int64_t* edge_from,
                           int64_t* node_from, double* cost3, int32_t* chosen) {
  SWE_GUARD_BEGIN
  if (strategy < SWE_REORDER_AUTO || strategy > SWE_REORDER_RCM)
    return fail(nullptr, SWE_ERR_INVALID_ARGUMENT, "unknown reorder strategy");
  swe_params p;
  swe_params_default(&p);
  HostInstance h;
  std::string why;
  swe_status st = read_instance(mesh, &p, &h, &why);
  if (st != SWE_OK) return fail(nullptr, st, why);
  why = swe::validate_instance(h);
  if (!why.empty()) return fail(nullptr, SWE_ERR_INVALID_MESH, why);
  double c3[3] = {0., 0., 0.};
  swe::Layout L;
  if (strategy == SWE_REORDER_AUTO) {
    L = swe::choose_layout(h, strategy, c3, nullptr);
  } else {
    L = swe::make_layout(h, strategy);
    c3[strategy] = swe::gather_sectors(swe::apply_layout(h, L));
  }
  if (cost3)
    for (int q = 0; q < 3; ++q) cost3[q] = c3[q];
  if (chosen) *chosen = L.strategy;
  auto emit = [&](int64_t* out, const std::vector<int64_t>& from, int64_t n) {
    if (!out) return;
    for (int64_t j = 0; j < n; ++j) out[j] = L.identity() ? j : from[j];
  };
  emit(cell_from, L.cell_from, h.C);
  emit(edge_from, L.edge_from, h.E);
  emit(node_from, L.node_from, h.N);
  return SWE_OK;
  SWE_GUARD_END(nullptr)
}

// ------------------------------------------------------------------ batched
swe_status swe_batch_create(int32_t n_instances, const swe_mesh* meshes, const double* const* prim0,
                            const swe_params* params, int32_t n_params, swe_batch** out) {
  Trace trace("swe_batch_create");
  SWE_GUARD_BEGIN
  if (!out) return fail(nullptr, SWE_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  if (n_instances <= 0 || !meshes || !prim0) return fail(nullptr, SWE_ERR_INVALID_ARGUMENT, "no instances");
  if (params && n_params != 1 && n_params != n_instances)
    return fail(nullptr, SWE_ERR_INVALID_ARGUMENT, "n_params must be 1 or n_instances");
  std::vector<HostInstance> inst(n_instances);
  std::vector<int> reorder(n_instances);
  swe_params p0;
  swe_params_default(&p0);
  if (params) p0 = params[0];
  std::string why;
  bool all_auto = true;
  int64_t total = 0;
  for (int q = 0; q < n_instances; ++q) {
    swe_params p = p0;
    if (params && n_params == n_instances) p = params[q];
    swe_status st = check_params(&p, &why);
    if (st != SWE_OK) return fail(nullptr, st, "instance " + std::to_string(q) + ": " + why);
    if (p.flux != p0.flux || p.wavespeed != p0.wavespeed)
      return fail(nullptr, SWE_ERR_UNSUPPORTED, "all instances of a batch must use the same flux and wave speed");
    if (!prim0[q]) return fail(nullptr, SWE_ERR_INVALID_ARGUMENT, "prim0[" + std::to_string(q) + "] is NULL");
    st = read_instance(&meshes[q], &p, &inst[q], &why);
    if (st == SWE_OK) {
      why = swe::validate_instance(inst[q]);
      if (!why.empty()) st = SWE_ERR_INVALID_MESH;
    }
    if (st != SWE_OK) return fail(nullptr, st, "instance " + std::to_string(q) + ": " + why);
    reorder[q] = p.reorder;
    all_auto = all_auto && p.reorder == SWE_REORDER_AUTO;
    total += inst[q].C;
  }
  std::unique_ptr<swe_batch> b;
  swe_status st;
  if (all_auto && total >= kTimedLayoutCells) {
    st = create_batch_timed(inst, p0, prim0, &b, &why);
  } else {
    std::vector<swe::Layout> lay(n_instances);
    st = SWE_OK;
    for (int q = 0; q < n_instances && st == SWE_OK; ++q) {
      st = lay_out(&inst[q], reorder[q], &lay[q], &why);
      if (st != SWE_OK) why = "instance " + std::to_string(q) + ": " + why;
    }
    if (st == SWE_OK) st = build_batch(std::move(inst), std::move(lay), p0, prim0, &b, &why);
  }
  if (st != SWE_OK) return fail(nullptr, st, why);
  *out = b.release();
  return SWE_OK;
  SWE_GUARD_END(nullptr)
}

swe_status swe_batch_destroy(swe_batch* b) {
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  cudaStreamSynchronize(b->eng.stream());
  delete b;
  return SWE_OK;
}

swe_status swe_batch_set_stream(swe_batch* b, void* stream) {
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  b->eng.set_stream(stream ? (cudaStream_t)stream : nullptr);
  return SWE_OK;
}

swe_status swe_batch_run_cfl(swe_batch* b, int32_t scheme, int64_t n_steps) {
  Trace trace("swe_batch_run_cfl");
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  if (!b->eng.has_scheme(scheme) || n_steps < 0) return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, "bad scheme or n_steps");
  cudaError_t e = b->eng.run_graph(scheme, 1, n_steps);
  if (e != cudaSuccess) return cuda_fail(&b->err, e, "swe_batch_run_cfl");
  return SWE_OK;
}

swe_status swe_batch_run(swe_batch* b, int32_t scheme, double dt, int64_t n_steps) {
  Trace trace("swe_batch_run");
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  if (!b->eng.has_scheme(scheme) || n_steps < 0) return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, "bad scheme or n_steps");
  if (!(dt > 0.) || !std::isfinite(dt)) return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, "dt must be positive and finite");
  const std::vector<double> dts((size_t)b->eng.I(), dt);  // the same dt for every instance
  cudaError_t e = cudaMemcpyAsync(b->eng.d_fixed_dt, dts.data(), dts.size() * sizeof(double), cudaMemcpyHostToDevice,
                                  b->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->eng.stream());
  if (e == cudaSuccess) e = b->eng.run_graph(scheme, 2, n_steps);
  if (e != cudaSuccess) return cuda_fail(&b->err, e, "swe_batch_run");
  return SWE_OK;
}

swe_status swe_batch_get_prim(swe_batch* b, int32_t q, double* prim_out) {
  if (!b || !prim_out || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  const int64_t c0 = b->eng.cell_off[q], n = b->eng.cell_off[q + 1] - c0;
  return download_prim(b->eng, prim_out, c0, n, &b->err);
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_adjoint_forward(swe_batch* b, int32_t scheme, int64_t n_steps, int64_t checkpoint_every,
                                     int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every,
                                     double* traces_out) {
  Trace trace("swe_batch_adjoint_forward");
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  if (!b->eng.has_scheme(scheme) || n_steps <= 0 || checkpoint_every <= 0 || n_gauges < 0 || obs_every <= 0)
    return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, "bad scheme, step counts or gauge count");
  if (n_gauges > 0 && (!gauge_cells || !traces_out))
    return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, "gauge_cells and traces_out are required");
  std::vector<int> g(n_gauges);
  for (int q = 0; q < n_gauges; ++q) {
    if (gauge_cells[q] < 0 || gauge_cells[q] >= b->eng.C())
      return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, "gauge cell out of range");
    g[q] = (int)device_cell(b->eng, gauge_cells[q]);
  }
  std::string e = b->eng.adjoint_forward(scheme, n_steps, checkpoint_every, g.data(), n_gauges, obs_every,
                                         traces_out);
  if (!e.empty()) return fail(&b->err, SWE_ERR_CUDA, e);
  return SWE_OK;
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_adjoint_backward(swe_batch* b, const double* trace_grads, double* grad_prim0,
                                      double* grad_bathymetry) {
  Trace trace("swe_batch_adjoint_backward");
  if (!b || !grad_prim0 || !grad_bathymetry) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  std::string e = adjoint_backward_caller(b->eng, trace_grads, grad_prim0, grad_bathymetry);
  if (!e.empty()) return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, e);
  return SWE_OK;
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_run_traces(swe_batch* b, int32_t scheme, int64_t n_steps, const double* dts, int32_t n_gauges,
                                const int64_t* gauge_cells, int64_t obs_every, double* traces_out) {
  Trace trace("swe_batch_run_traces");
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return run_traces_common(b->eng, &b->err, scheme, n_steps, dts, n_gauges, gauge_cells, obs_every, traces_out);
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_set_bathymetry(swe_batch* b, const double* const* z) {
  Trace trace("swe_batch_set_bathymetry");
  if (!b || !z) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return set_bathymetry_common(b->eng, &b->err, std::vector<const double*>(z, z + b->eng.I()));
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_prime(swe_batch* b) {
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return prime(b->eng, &b->err);
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_set_prim_device(swe_batch* b, int32_t q, const double* in) {
  if (!b || !in || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  Engine& g = b->eng;
  const int64_t c0 = g.cell_off[q], n = g.cell_off[q + 1] - c0;
  k_unpack<<<(int)((n + 255) / 256), 256, 0, g.stream()>>>(in, g.state(0, 0) + c0, g.state(0, 1) + c0,
                                                            g.state(0, 2) + c0, (int)n, nullptr,
                                                            g.d_cell_from ? g.d_cell_from + c0 : nullptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(&b->err, e, "swe_batch_set_prim_device");
  return SWE_OK;
}

swe_status swe_batch_adjoint_forward_device(swe_batch* b, int32_t scheme, int64_t n_steps, int64_t checkpoint_every,
                                            int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every,
                                            double* traces_out) {
  Trace trace("swe_batch_adjoint_forward_device");
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  return adjoint_forward_device_common(b->eng, &b->err, scheme, n_steps, checkpoint_every, n_gauges, gauge_cells,
                                       obs_every, traces_out);
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_adjoint_backward_device(swe_batch* b, const double* trace_grads, double* grad_prim0,
                                             double* grad_bathymetry) {
  Trace trace("swe_batch_adjoint_backward_device");
  if (!b || !grad_prim0 || !grad_bathymetry) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  std::string e = b->eng.adjoint_backward(trace_grads, grad_prim0, grad_bathymetry, true);
  if (!e.empty()) return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, e);
  return SWE_OK;
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_adjoint_prepare(swe_batch* b) {
  Trace trace("swe_batch_adjoint_prepare");
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  std::string e = b->eng.adjoint_init();
  if (!e.empty()) return fail(&b->err, SWE_ERR_CUDA, e);
  return SWE_OK;
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_adjoint_set_regularisation(swe_batch* b, double depth) {
  if (!b || !(depth >= 0.) || !std::isfinite(depth)) return SWE_ERR_INVALID_ARGUMENT;
  b->eng.set_adjoint_regularisation(depth);
  return SWE_OK;
}

swe_status swe_batch_adjoint_dts(swe_batch* b, double* dts_out) {
  if (!b || !dts_out) return SWE_ERR_INVALID_ARGUMENT;
  std::string e = b->eng.adjoint_dts(dts_out);
  if (!e.empty()) return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, e);
  return SWE_OK;
}

swe_status swe_batch_integrals(swe_batch* b, int32_t q, double* out3) {
  Trace trace("swe_batch_integrals");
  if (!b || !out3 || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  const int64_t c0 = b->eng.cell_off[q], n = b->eng.cell_off[q + 1] - c0;
  cudaError_t e = b->eng.integrals(c0, n, out3);
  if (e != cudaSuccess) return cuda_fail(&b->err, e, "swe_batch_integrals");
  return SWE_OK;
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_set_scheme(swe_batch* bt, int32_t n_stages, const double* a, const double* b,
                                const double* c) {
  if (!bt) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  swe::Scheme sc;
  std::string e = make_scheme(n_stages, a, b, c, &sc);
  if (!e.empty()) return fail(&bt->err, SWE_ERR_INVALID_ARGUMENT, e);
  bt->eng.set_custom_scheme(sc);
  return SWE_OK;
  SWE_GUARD_END(&bt->err)
}

swe_status swe_batch_get_tuning(swe_batch* b, int32_t q, int32_t* out4) {
  if (!b || !out4 || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  out4[0] = b->eng.layouts.empty() ? 0 : b->eng.layouts[q].strategy;
  for (int k = 0; k < 3; ++k) out4[1 + k] = b->eng.blocks()[k];
  return SWE_OK;
}

swe_status swe_batch_time(swe_batch* b, int32_t q, double* t) {
  if (!b || !t || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaMemcpyAsync(t, b->eng.work().tsum + q, sizeof(double), cudaMemcpyDeviceToHost, b->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->eng.stream());
  if (e != cudaSuccess) return cuda_fail(&b->err, e, "swe_batch_time");
  return SWE_OK;
}

swe_status swe_batch_set_time(swe_batch* b, int32_t q, double t) {
  if (!b || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  if (!std::isfinite(t)) return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, "t must be finite");
  cudaError_t e =
      cudaMemcpyAsync(b->eng.work().tsum + q, &t, sizeof(double), cudaMemcpyHostToDevice, b->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->eng.stream());
  if (e != cudaSuccess) return cuda_fail(&b->err, e, "swe_batch_set_time");
  return SWE_OK;
}

swe_status swe_batch_min_len_to_wavespeed(swe_batch* b, int32_t q, double* r) {
  if (!b || !r || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  unsigned long long k = 0;
  cudaError_t e = cudaMemcpyAsync(&k, b->eng.work().r + q, sizeof(k), cudaMemcpyDeviceToHost, b->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->eng.stream());
  if (e != cudaSuccess) return cuda_fail(&b->err, e, "swe_batch_min_len_to_wavespeed");
  *r = swe::order_val(k);
  return SWE_OK;
}

swe_status swe_batch_set_min_len_to_wavespeed(swe_batch* b, int32_t q, double r) {
  if (!b || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  if (!(r > 0.) || !std::isfinite(r)) return fail(&b->err, SWE_ERR_INVALID_ARGUMENT, "r must be positive and finite");
  const unsigned long long k = swe::order_key(r);
  cudaError_t e = cudaMemcpyAsync(b->eng.work().r + q, &k, sizeof(k), cudaMemcpyHostToDevice, b->eng.stream());
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->eng.stream());
  if (e != cudaSuccess) return cuda_fail(&b->err, e, "swe_batch_set_min_len_to_wavespeed");
  return SWE_OK;
}

swe_status swe_batch_set_prim(swe_batch* b, int32_t q, const double* prim_in) {
  if (!b || !prim_in || q < 0 || q >= b->eng.I()) return SWE_ERR_INVALID_ARGUMENT;
  SWE_GUARD_BEGIN
  const int64_t c0 = b->eng.cell_off[q], n = b->eng.cell_off[q + 1] - c0;
  return upload_prim(b->eng, prim_in, c0, n, &b->err);
  SWE_GUARD_END(&b->err)
}

swe_status swe_batch_launch_count(swe_batch* b, int64_t* n) {
  if (!b || !n) return SWE_ERR_INVALID_ARGUMENT;
  *n = b->eng.launches();
  return SWE_OK;
}

swe_status swe_batch_synchronize(swe_batch* b) {
  if (!b) return SWE_ERR_INVALID_ARGUMENT;
  return check_device(b->eng, &b->err);
}

const char* swe_batch_last_error(swe_batch* b) {
  if (!b) return g_create_error.c_str();
  return b->err.c_str();
}

}  // extern "C"
