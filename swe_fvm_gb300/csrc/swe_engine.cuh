// swe_engine.cuh -- device data layout and the engine that owns it.
//
// Layout in HBM (all indices int32, all values FP64, structure of arrays):
//   cells  : C = sum of the instances' cells, concatenated instance by instance
//   edges  : E, likewise; nodes: N, likewise
//   "slot" (i, k) = interface value of cell i on its local edge k, stored at
//   k * C + i, so a warp writes and reads its own cells' slots coalesced.
// Static per-cell records hold every quantity of the reference step that
// depends on the mesh alone (precomputed once on the host with the reference's
// operation order); the kernels do only state-dependent arithmetic.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "swe_physics.cuh"

namespace swe {

constexpr int kComboStride = 12;  // doubles per full-wet combination record
constexpr int kPw1Stride = 12;    // doubles per PartWet1 record
constexpr int kDryStride = 8;     // doubles per dry-cell record

enum : unsigned { kErrNonFinite = 1u, kErrBadState = 2u, kErrBadIndex = 4u };

// The full-wet combination records are stored combination-major, [8][C][12]:
// the record of cell i for neighbour combination `mask` starts here.  Nearly
// every fully-wet cell has only fully-wet neighbours (mask 0), so the records
// a warp reads are contiguous.
__host__ __device__ __forceinline__ size_t combo_off(int C, int i, int mask) {
  return ((size_t)mask * (size_t)C + (size_t)i) * kComboStride;
}

// Static per-slot record read by the update kernel with two 16-byte loads:
// L(e_k) / A, the edge-centre bathymetry and the normal times L(e_k) / A.
struct __align__(16) SlotRec {
  double cek, ze, nxc, nyc;
};

// Static per-edge record read by the flux kernel with three 16-byte loads:
// the owner's outward normal and tangent, the edge-centre bathymetry and
// min(2 A_owner / L, 2 A_neighbour / L).
struct __align__(16) EdgeRec {
  double nx, ny, tx, ty, b, lmin;
};

// PartWet2 (src/MUSCLObject.cpp:114-191) geometry: vertices sorted by z.
struct Pw2Rec {
  double p[3][3];     // sorted vertices (x, y, z), lowest first
  double ratio_b;     // (b12 - b23) / (b13 - b23)
  double hd2f;        // 2 b13 - b12 - b23
  double d13;         // b13 - b23
  double beta;        // (b13 - b12) / (b13 - b23)
  double tp0x, tp0y;  // T - P_lowest
  double dnode[3][2]; // P_k - T, cell node order
  double dedge[3][2]; // E_k - T, cell edge order
  int lo;             // global id of the lowest node
  int flat;           // b13 - b23 < tol
  int sk[3];          // local (cell-order) index of each sorted vertex
  int pad;
};

struct DevMesh {
  int C, E, N, I;
  // cells
  const int* cnode;           // [3][C]
  const int* cnbr;            // [3][C], -1 = wall
  const int* cedge;           // [3][C]
  const unsigned char* cown;  // [C] bit k: this cell owns edge k
  const double* bc;           // [C] centroid bathymetry
  const double* fwthr;        // [C] max node z, +inf for boundary cells
  const double* area;         // [C]
  const double* zn;           // [3][C] node z
  const double* ze;           // [3][C] edge-centre z
  const double* cek;          // [3][C] L(e_k) / A
  const double* cnxc;         // [3][C] outward normal of edge k times L_k / A (x)
  const double* cnyc;         // [3][C] (y)
  const double* dry;          // [C][8] dry-cell node/edge values and slope
  const double* combo;        // [8][C][12] full-wet plane records (combo_off)
  const double* pw1;          // [C][12]
  const Pw2Rec* pw2;          // [C]
  const int* cinst;           // [C] instance of the cell (batched only)
  const SlotRec* srec;        // [3][C] cek, ze, cnxc, cnyc of each slot, packed
  const int2* cslot;          // [3][C] (cedge, cnbr) of each slot, packed
  // edges
  const int* eown;    // [E]
  const int* enb;     // [E] -1 = wall
  const int* eslotl;  // [E] slot of the owner's interface value
  const int* eslotr;  // [E] slot of the neighbour's interface value
  const double* enx;
  const double* eny;
  const double* etx;
  const double* ety;
  const double* ezm;    // edge-centre bathymetry
  const double* elmin;  // min(2A_owner/L, 2A_nb/L)
  const int* einst;     // [E] (batched only)
  const EdgeRec* erec;  // [E] enx, eny, etx, ety, ezm, elmin, packed
  const int4* eidx;     // [E] (eown, enb, eslotl, eslotr), packed
  // nodes
  const double* nz;     // [N]
  const int* nptr;      // [N+1] the cells around each node (CSR) ...
  const int* ncell;     // [3C]  ... as (cell << 2) | local node index
  // instances
  const int* inst_cell_begin;  // [I]
  const double* inst_cfl;      // [I]
  const double* inst_cor;      // [I]
  // the engine's device error word (DevWork::err), for the range checks of
  // checked builds in code that sees only the mesh
  unsigned* err;
};

struct DevWork {
  double* ew;  // [3][C] interface w
  double* eu;
  double* ev;
  double* sx;  // [3][C] source gradient
  double* sy;
  double* f0;  // [E] fluxes
  double* f1;
  double* f2;
  double* drain;               // [C] draining time step
  unsigned long long* maxwp;   // [N] ordered keys of the node maxima
  int* pwlist;                 // [C] partially-wet cells of this stage
  int* pwcount;                // [1]
  double* pwrec;               // [C] PartWet1 level of listed cells
  // [C] pass-1 class of each cell: type (0 dry, 1 partially wet, 2 fully wet)
  // | neighbour combination mask << 2 | combination plane kept << 5
  unsigned char* cls;
  double* ftape;               // [7][E] flux intermediates kept for the adjoint, or null
  unsigned long long* r;       // [I] ordered key of min length-to-wavespeed
  double* dt;                  // [I] step dt
  double* tsum;                // [I] accumulated time
  const double* fixed_dt;      // [I] dt for fixed-step runs
  unsigned* err;               // [1] error bits
};

// A gathered index.  In checked builds (-DSWE_CHECKED, build(checked=True))
// an index outside [0, n) sets kErrBadIndex and becomes 0, so the access stays
// in bounds and the kernel's control flow (and its warp collectives) is
// unchanged; the product build returns the index untouched.
__device__ __forceinline__ int gidx(unsigned* err, int idx, int n) {
#ifdef SWE_CHECKED
  if ((unsigned)idx >= (unsigned)n) {
    atomicOr(err, kErrBadIndex);
    return 0;
  }
#else
  (void)err;
  (void)n;
#endif
  return idx;
}
__device__ __forceinline__ int gidx(const DevWork& wk, int idx, int n) { return gidx(wk.err, idx, n); }
__device__ __forceinline__ int gidx(const DevMesh& m, int idx, int n) { return gidx(m.err, idx, n); }

// One Runge-Kutta stage in Shu-Osher form (src/Solvers.cpp:5-59).
struct Stage {
  bool first;     // U = U0.cons + RHS(dt)
  double a, b, c; // U = a U0.cons + b Uprev.cons + RHS(c dt)
};

constexpr int kMaxStages = 4;
constexpr int kCustomScheme = 3;  // id of the caller-defined table
struct Scheme {
  int n;
  Stage s[kMaxStages];
};
// Built-in schemes 0 Euler, 1 SSPRK2, 2 SSPRK3.
Scheme scheme_table(int scheme);

// Host-side description of one instance after validation.
struct HostInstance {
  int64_t C, E, N;
  std::vector<double> geom;
  std::vector<int64_t> en, ec, cn, ce, ct;
  double cfl, cor;
};

// Order of an instance's cells, edges and nodes on the device
// (swe_layout.cuh builds them).
enum : int { kLayoutAuto = -1, kLayoutKeep = 0, kLayoutMorton = 1, kLayoutRcm = 2 };
struct Layout {
  int strategy = kLayoutKeep;
  // device position -> the caller's index (empty when strategy is kLayoutKeep)
  std::vector<int64_t> cell_from, edge_from, node_from;
  // the caller's cell index -> device position
  std::vector<int64_t> cell_to;
  bool identity() const { return strategy == kLayoutKeep; }
};

struct AdjWork;
struct AdjointState;
void adjoint_state_delete(AdjointState* a);

class Engine {
 public:
  Engine() = default;
  ~Engine();
  // Validates and precomputes every instance, uploads, allocates work arrays.
  // Returns an empty string on success, else the error message (status in *st).
  // block > 0 fixes the threads per block of every cell and edge kernel.
  std::string init(std::vector<HostInstance>&& inst, int flux, int ws, int block, int* st, bool batched);

  // Time schemes: 0..2 built in, kCustomScheme once set_custom_scheme defined
  // it.  Changing the custom table drops its captured step graphs.
  void set_custom_scheme(const Scheme& sc);
  bool has_scheme(int id) const { return (id >= 0 && id <= 2) || (id == kCustomScheme && custom_.n > 0); }
  Scheme scheme_of(int id) const { return id == kCustomScheme ? custom_ : scheme_table(id); }

  // Threads per block of the reconstruction kernels (k_recon1, k_recon2), the
  // edge-flux kernel (k_flux) and the drain/update kernels; drops the
  // captured step graphs when they change.
  void set_blocks(const int blocks[3]);
  const int* blocks() const { return blk_; }
  // Times steps of `scheme` with 64, 128 and 256 threads per block and keeps
  // the fastest per kernel group.  The state, the accumulated time and the
  // error word are restored; the caller re-primes the flux pass.  Choices are
  // cached per (device, flux, wave speed, batched, Coriolis, scheme,
  // log2 of the cell count) for the life of the process.
  cudaError_t autotune_blocks(int scheme);
  // Cell layouts of the instances (device position -> caller's index) and
  // their device copies over the concatenated cells: d_cell_from (global
  // device position -> the caller's local row) and d_cell_to (global caller
  // row -> global device position); both null when every instance keeps the
  // caller's order.
  std::vector<Layout> layouts;
  int* d_cell_from = nullptr;
  int* d_cell_to = nullptr;
  std::string set_layouts(std::vector<Layout>&& lay);
  // Replaces the node bathymetry of the instances whose pointer is not null
  // (each in the caller's node order, N_q values), recomputes every mesh record
  // with the same device order and re-uploads them into the same buffers (the
  // captured step graphs stay valid); drops the adjoint's tape.  The state is
  // kept; the caller re-primes the flux pass.
  std::string set_bathymetry(const std::vector<const double*>& z);
  // Mean ms of one graph-replayed step of `scheme` (CFL dt) over n steps after
  // one warm-up replay, run from the current state, which is then restored
  // with the accumulated time, the step dt and the error word (the caller
  // re-primes the flux pass).
  cudaError_t time_steps(int scheme, int n, float* ms);
  // Device bytes this engine allocated.
  size_t device_bytes() const { return bytes_; }

  // NULL selects the engine's own non-blocking stream.
  // Work already enqueued on the previous stream is ordered before anything
  // enqueued on the new one (an event recorded on the old stream, waited on
  // by the new one).
  void set_stream(cudaStream_t s);
  cudaStream_t stream() const { return stream_; }

  // Resets the node maxima and the part-wet list (done by k_drain at the end
  // of every stage; needed before a standalone reconstruction).
  cudaError_t reset_pass();
  // Launches one reconstruction (pass 1 + pass 2) and one flux pass.
  cudaError_t interface_values(const double* W, const double* U, const double* V, int latch_mode);
  cudaError_t fluxes(const double* W);
  // One whole step of `scheme`; latch_mode 1 = CFL dt, 2 = fixed dt from
  // work.fixed_dt.  Enqueued on the engine's stream.
  cudaError_t step(int scheme, int latch_mode);
  // n steps through a cached CUDA graph of one step.
  cudaError_t run_graph(int scheme, int latch_mode, int64_t n);
  // One step launched kernel by kernel with CUDA events between them;
  // adds the durations (ms) of k_recon1, k_recon2, k_flux, k_drain, k_update
  // to acc[0..4] and the whole step to acc[5].  Synchronises.
  cudaError_t step_timed(int scheme, int latch_mode, double* acc);

  // Discrete adjoint (swe_adjoint.cu): reverse of one stage whose input is
  // `in` and whose step started from `u0`, given aw.lam; accumulates aw.lamp,
  // aw.lam0, aw.lz.
  cudaError_t adjoint_stage_reverse(const Stage& st, const double* const* in, const double* const* u0, AdjWork& aw);
  cudaError_t adjoint_stage_reverse_stored(const Stage& st, const double* const* in, const double* const* u0,
                                           AdjWork& aw, const DevWork& wk, const double* nst);
  // volume, kinetic and potential energy of cells c0 .. c0+n-1 (host out[3])
  cudaError_t integrals(int64_t c0, int64_t n, double* out_host);
  // the update kernel of one stage alone (the rest of the stage already ran),
  // also keeping the state before ConsAssigner in nst [3][C]
  cudaError_t update_only(const Stage& st, const double* const* in, const double* const* u0, double* const* out,
                          double* nst);
  // The adjoint's one-time tables and work arrays (node and twin lists, plane
  // adjoints); a no-op once built.  Returns "" or an error message.
  std::string adjoint_init();
  // Taped forward run for the adjoint: n_steps CFL steps from the current
  // state, checkpoint every ckpt steps, w at the gauge cells every obs steps
  // into traces_host (n_steps / obs rows).  Returns "" or an error message.
  // traces_device: traces_host is a device pointer (the traces are copied on
  // the device).
  std::string adjoint_forward(int scheme, int64_t n_steps, int64_t ckpt, const int* gauges, int n_gauges,
                              int64_t obs, double* traces_host, bool traces_device = false);
  // n_steps steps of `scheme` with the given dts (n_steps x I, step-major),
  // w at the gauge cells after every obs-th step into traces (n_steps / obs
  // rows); no tape.  Returns "" or an error message.
  std::string run_traces(int scheme, int64_t n_steps, const double* dts_host, const int* gauges, int n_gauges,
                         int64_t obs, double* traces_host);
  // Reverse of the taped run: trace_grads (n_obs x n_gauges) are the adjoints
  // of the traces; returns the gradient with respect to the initial primitive
  // state (3 x C interleaved) and the node bathymetry (N).
  // device: every pointer is device memory and the gradients are written in
  // the caller's cell and node order.
  std::string adjoint_backward(const double* trace_grads_host, double* grad_prim_host, double* grad_z_host,
                               bool device = false);
  std::string adjoint_dts(double* out_host);
  // Depth below which the reverse regularises the w-slope of a PartWet1 level
  // that feeds a node maximum (kEta1 by default; 0 = exact derivative).
  void set_adjoint_regularisation(double depth) { adj_reg_depth_ = depth; }

  int C() const { return mesh_.C; }
  int E() const { return mesh_.E; }
  int N() const { return mesh_.N; }
  int I() const { return mesh_.I; }
  int64_t launches() const { return launches_; }
  double* state(int buf, int comp) { return state_[buf * 3 + comp]; }
  const DevWork& work() const { return work_; }
  DevWork& work() { return work_; }
  const DevMesh& mesh() const { return mesh_; }

  // Instance ranges in the concatenated arrays.
  std::vector<int64_t> cell_off, edge_off, node_off;
  // Host copies of the per-instance topology needed by the layout getters.
  std::vector<HostInstance> host;
  // global device cell / node position -> global caller index, built on first
  // use by the device-memory adjoint outputs
  int* d_cell_caller = nullptr;
  int* d_node_caller = nullptr;
  std::string caller_maps();
  double* d_io = nullptr;        // [3C] staging buffer for the interleaved 3 x C field
  unsigned* d_ioflag = nullptr;  // non-finite flag of the last upload
  double* d_fixed_dt = nullptr;  // [I] device dt of fixed-step runs
  double* h_fixed_dt = nullptr;  // pinned host scalar

 private:
  cudaError_t launch_stage(const Stage& st, const double* const* in, const double* const* u0, double* const* out,
                           bool first_stage_of_step, int latch_mode, cudaEvent_t* ev = nullptr);
  template <class T>
  T* dalloc(size_t n);

  DevMesh mesh_{};
  DevWork work_{};
  double* state_[6] = {};
  std::vector<void*> allocs_;
  cudaStream_t stream_ = nullptr;
  cudaStream_t own_stream_ = nullptr;
  // second stream of a stage: PartWet2 and the fluxes of the edges next to
  // partially-wet cells run on it while the other edges' fluxes run on stream_
  cudaStream_t side_ = nullptr;
  cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
  int flux_ = 1, ws_ = 2;
  int blk_[3] = {256, 256, 256};  // reconstruction, edge flux, drain/update
  bool batched_ = false;
  bool cor0_ = true;  // every instance has cor = 0: no Coriolis arithmetic in the reconstruction
  double* d_integrals_ = nullptr;  // partial sums of the integrals
  void launch_recon1(const double* W, const double* U, const double* V, int latch_mode);
  void launch_recon2(const double* W, const double* U, const double* V, cudaStream_t s);
  // fluxes: mode 0 every edge; mode 1 the edges with no partially-wet cell;
  // fluxes_pw: the others (those of the listed cells), on stream s
  cudaError_t fluxes(const double* W, int mode);
  void fluxes_pw(const double* W, cudaStream_t s);
  void launch_update(const Stage& st, const double* const* in, const double* const* u0, double* const* out,
                     double* nst);
  int64_t launches_ = 0;
  size_t bytes_ = 0;
  // copy of the state (3 x C) to or from buf; after a restore also zeroes the
  // accumulated time, the step dt and the error word
  cudaError_t snapshot(double* buf, bool restore);
  cudaGraphExec_t graphs_[4][3] = {};  // [scheme id][latch mode]
  Scheme custom_{};
  AdjointState* adj_ = nullptr;
  std::vector<std::pair<void*, size_t>> mesh_arrays_;  // device mesh records in upload order
  double adj_reg_depth_ = kEta1;
};

// Precompute (swe_precompute.cu): fills the host images of DevMesh arrays for
// instance `inst` at offsets (c0, e0, n0) of the concatenated arrays.
struct HostImage {
  int C, E, N, I;
  std::vector<int> cnode, cnbr, cedge, cinst, eown, enb, eslotl, eslotr, einst, inst_cell_begin, nptr, ncell;
  std::vector<unsigned char> cown;
  std::vector<double> bc, fwthr, area, zn, ze, cek, cnxc, cnyc, dry, combo, pw1, enx, eny, etx, ety, ezm, elmin, nz,
      inst_cfl, inst_cor;
  std::vector<Pw2Rec> pw2;
  std::vector<SlotRec> srec;
  std::vector<int2> cslot;
  std::vector<EdgeRec> erec;
  std::vector<int4> eidx;
  void resize(int C_, int E_, int N_, int I_);
};
std::string validate_instance(const HostInstance& h);
void precompute_instance(const HostInstance& h, int inst, int64_t c0, int64_t e0, int64_t n0, HostImage& img);

}  // namespace swe
