/*
 * swe_fvm_gb300.h -- C ABI of the GB300 explicit finite-volume shallow-water
 * step (FP64, unstructured triangles, wet/dry MUSCL + HLL/HLLC + SSP-RK).
 *
 * One `swe_ctx` is the device-resident counterpart of the reference's
 * SpaceDisc + TimeDisc pair (include/SpaceDisc.h:20-48, include/TimeDisc.h:4-23
 * of NikitaMatckevich/SWE_FVM); `swe_step` is one call of
 * Solvers::Euler / SSPRK2 / SSPRK3 (include/Solvers.h:6-8).  A `swe_batch`
 * holds many independent instances stepped together.
 *
 * Conventions
 *   - Arrays are the reference's layouts, host memory unless a name ends in
 *     `_device`.  Geometry: 3 x N column-major doubles (node i's x, y, z at
 *     [3i, 3i+1, 3i+2]; z is the bathymetry).  Topology: int64 row-major
 *     edge_nodes E x 2, edge_cells E x 2 (owner, neighbour or -1 = solid wall),
 *     cell_nodes / cell_edges / cell_neighbours C x 3.  Primitive state: 3 x C
 *     column-major (w, u, v) per cell, w = free-surface level.
 *   - The library copies every input; callers may free them after the call
 *     (the reference keeps references: include/TriangMesh.h:56-64).
 *   - Every function returns a swe_status; on failure the message is in
 *     swe_last_error(ctx) (or swe_last_error(NULL) for a failed create).
 *   - A context is not thread-safe (the reference is single-threaded);
 *     distinct contexts may run concurrently on distinct streams.
 *   - All state lives on the current CUDA device at create time.
 */
#ifndef SWE_FVM_GB300_H
#define SWE_FVM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error classes.  Replaces the reference's exceptions DomainError / SolverError
 * (include/Exceptions.h:4-10) and std::runtime_error (include/Assigners.h:20). */
typedef enum swe_status {
  SWE_OK = 0,
  SWE_ERR_INVALID_ARGUMENT = 1,
  SWE_ERR_INVALID_MESH = 2, /* bad index, non-manifold edge, boundary code other than -1 */
  SWE_ERR_NONFINITE = 3,    /* non-finite state detected on the device */
  SWE_ERR_TIMEOUT = 4,      /* a bounded device wait gave up */
  SWE_ERR_CUDA = 5,
  SWE_ERR_OUT_OF_MEMORY = 6,
  SWE_ERR_UNSUPPORTED = 7
} swe_status;

/* Flux plugin: Fluxes::HLL<W> / Fluxes::HLLC<W> (include/Fluxes.h:14-111). */
typedef enum swe_flux { SWE_FLUX_HLL = 0, SWE_FLUX_HLLC = 1 } swe_flux;
/* Wave-speed plugin: Wavespeeds::Rusanov / Davis / Einfeldt (src/Fluxes.cpp:5-26). */
typedef enum swe_wavespeed { SWE_WS_RUSANOV = 0, SWE_WS_DAVIS = 1, SWE_WS_EINFELDT = 2 } swe_wavespeed;
/* Device order of an instance's cells, edges and nodes.  The reference has
 * one order, the caller's (include/TriangMesh.h:14-65); every array crossing
 * this boundary stays in the caller's order whatever the device uses, and
 * states are bit-identical in every order (each cell and edge is computed
 * from its own topology row).  MORTON sorts cells by the z-order of their
 * centroids, RCM by reverse Cuthill-McKee over the cell-neighbour graph;
 * edges follow their owner cell, nodes their first cell.  AUTO (the default)
 * picks one of KEEP, MORTON, RCM: for meshes of 65,536 cells or more
 * swe_create builds a context in each order and keeps the one whose SSPRK2
 * steps run fastest (the caller's order unless another is more than 2 %
 * faster), and so does swe_batch_create for batches of 65,536 cells or more
 * whose instances all ask for AUTO (one order for every instance); smaller
 * meshes and batches take, per instance, the one with the fewest 32-byte
 * sectors gathered per warp (the caller's order unless another saves more
 * than 5 %). */
typedef enum swe_reorder {
  SWE_REORDER_AUTO = -1,
  SWE_REORDER_KEEP = 0,
  SWE_REORDER_MORTON = 1,
  SWE_REORDER_RCM = 2
} swe_reorder;
/* Time scheme: Solvers::Euler / SSPRK2 / SSPRK3 (src/Solvers.cpp:5-59). */
typedef enum swe_scheme {
  SWE_SCHEME_EULER = 0,
  SWE_SCHEME_SSPRK2 = 1,
  SWE_SCHEME_SSPRK3 = 2,
  SWE_SCHEME_CUSTOM = 3 /* the table given to swe_set_scheme */
} swe_scheme;

/* Mesh in the reference's arrays (Topology + Domain geometry). */
typedef struct swe_mesh {
  int64_t num_nodes;
  int64_t num_edges;
  int64_t num_cells;
  const double* geometry;         /* 3 x num_nodes, column-major */
  const int64_t* edge_nodes;      /* num_edges x 2 */
  const int64_t* edge_cells;      /* num_edges x 2 */
  const int64_t* cell_nodes;      /* num_cells x 3 */
  const int64_t* cell_edges;      /* num_cells x 3 */
  const int64_t* cell_neighbours; /* num_cells x 3 */
} swe_mesh;

/* Physical and numerical parameters.  Defaults (swe_params_default) are the
 * reference's: HLLC + Einfeldt, cor = tau = 0 (SpaceDisc ctor,
 * include/SpaceDisc.h:24), CFL coefficient 0.15 (include/TimeDisc.h:22). */
typedef struct swe_params {
  int32_t flux;      /* swe_flux */
  int32_t wavespeed; /* swe_wavespeed */
  double cor;        /* Coriolis parameter (SpaceDisc::m_cor) */
  double tau;        /* friction (stored, unused by the reference: src/TimeDisc.cpp:38-39) */
  double cfl;        /* TimeDisc::CFLdt() = cfl * min length-to-wavespeed ratio */
  int32_t reorder;   /* swe_reorder: device order of cells, edges and nodes (default AUTO) */
  int32_t block;     /* threads per block of the cell and edge kernels: 0 = timed at creation
                        (default), else a multiple of 32 from 32 to 256 */
} swe_params;

typedef struct swe_ctx swe_ctx;
typedef struct swe_batch swe_batch;

/* Fills *p with the reference defaults. */
swe_status swe_params_default(swe_params* p);

/* Builds a context: validates and copies the mesh, precomputes the static
 * geometry on the host, uploads it and the initial primitive state (3 x C).
 * Replaces Topology(...) + Domain(...) + SpaceDisc(fluxer, domain, v0, cor, tau)
 * + TimeDisc(&sd) (include/TriangMesh.h:27-40, src/Bathymetry.cpp:6-8,
 * src/SpaceDisc.cpp:4-13, include/TimeDisc.h:6-7). */
swe_status swe_create(const swe_mesh* mesh, const double* prim0, const swe_params* params, swe_ctx** out);
swe_status swe_destroy(swe_ctx* ctx);

/* Runs kernels of this context on `stream` (a cudaStream_t; NULL = the
 * context's own stream).  Work already enqueued on the previous stream is
 * ordered before anything enqueued on the new one; swe_create returns with
 * its own device work finished.  The caller keeps `stream` alive while the
 * context uses it. */
swe_status swe_set_stream(swe_ctx* ctx, void* stream);

/* One time step of the scheme with a fixed dt: Solvers::X(&td, dt)
 * (src/Solvers.cpp:5-59).  Asynchronous on the context's stream. */
swe_status swe_step(swe_ctx* ctx, int32_t scheme, double dt);

/* n_steps fixed-dt steps, replayed from a captured CUDA graph. */
swe_status swe_run(swe_ctx* ctx, int32_t scheme, double dt, int64_t n_steps);

/* n_steps steps with dt = TimeDisc::CFLdt() taken before every step from the
 * previous flux pass (include/TimeDisc.h:13), all on the device.  If
 * t_elapsed is not NULL it receives the sum of the dts (synchronises). */
swe_status swe_run_cfl(swe_ctx* ctx, int32_t scheme, int64_t n_steps, double* t_elapsed);

/* TimeDisc::CFLdt() (include/TimeDisc.h:13); synchronises. */
swe_status swe_cfl_dt(swe_ctx* ctx, double* dt);
/* SpaceDisc::GetMinLenToWavespeed() of the last flux pass (include/SpaceDisc.h:31). */
swe_status swe_min_len_to_wavespeed(swe_ctx* ctx, double* r);

/* SpaceDisc::ComputeInterfaceValues() / ComputeFluxes() (src/SpaceDisc.cpp:33-74)
 * on the current state, for inspection with the getters below. */
swe_status swe_compute_interface_values(swe_ctx* ctx);
swe_status swe_compute_fluxes(swe_ctx* ctx);

/* Primitive state, 3 x C column-major in the caller's cell order
 * (VolumeField, include/ValueField.h:31-48).  Synchronous.  Setting the state
 * leaves the CFL ratio of the last flux pass in place, as assigning the
 * reference's volume field does. */
swe_status swe_get_prim(swe_ctx* ctx, double* prim_out);
swe_status swe_set_prim(swe_ctx* ctx, const double* prim_in);
/* Same, from / to device memory in the caller's order, asynchronous on the
 * context's stream. */
swe_status swe_get_prim_device(swe_ctx* ctx, double* prim_out_device);
swe_status swe_set_prim_device(swe_ctx* ctx, const double* prim_in_device);

/* Interface values and source gradients in the reference's EdgeField layout:
 * 3 x 2E column-major, slot 2e + (from < to) (include/ValueField.h:70-75);
 * row 0 of `src` is unused by the reference and returned as 0.  Either pointer
 * may be NULL.  Synchronous. */
swe_status swe_get_edge_values(swe_ctx* ctx, double* edg_out, double* src_out);
/* Edge fluxes, 3 x E (SpaceDisc::GetFluxes, include/SpaceDisc.h:28). */
swe_status swe_get_fluxes(swe_ctx* ctx, double* flux_out);
/* Node maxima of the reconstructed level after pass 1 of the last
 * reconstruction (MUSCLObject::m_max_wp, include/MUSCLObject.h:68), N values. */
swe_status swe_get_node_max(swe_ctx* ctx, double* max_out);

/* Profiling: runs `reps` steps of `scheme` (CFL dt) launching the stage
 * kernels one by one with CUDA events between them on the context's stream.
 * out_ms[0..4] = mean duration of one launch of the reconstruction pass 1,
 * pass 2, flux, draining-time-step and update kernels; out_ms[5] = mean step
 * time.  Advances the state; synchronises.  No reference counterpart. */
swe_status swe_time_kernels(swe_ctx* ctx, int32_t scheme, int64_t reps, double* out_ms);

/* FP64 FMA throughput of the current device in TFLOP/s (best of 5 timed
 * launches of independent FMA chains): the arithmetic ceiling of the step.
 * No reference counterpart. */
swe_status swe_measure_fp64_peak(double* tflops);

/* Compares the integer-pipe FP64 division and square root used by the kernels
 * with the hardware instructions on n pseudo-random operands (all classes:
 * normal, near-power-of-two significands, extreme exponents, specials) and
 * returns the number of results that differ in any bit.  No reference
 * counterpart. */
swe_status swe_selftest_fp64(int64_t n, uint64_t seed, int64_t* div_mismatches, int64_t* sqrt_mismatches);

/* Compares the hand-written reverse of the flux plugin (flux, wavespeed) with
 * its forward-mode Jacobian on n random interface states (some with a dry
 * side) and returns the largest normwise relative difference of the
 * 7-component adjoint (max |hand - dual| / max |dual|).  No
 * reference counterpart. */
swe_status swe_selftest_flux_adjoint(int32_t flux, int32_t wavespeed, int64_t n, uint64_t seed, double* max_rel_err);

/* Size and counters. */
swe_status swe_num_cells(swe_ctx* ctx, int64_t* n);
/* Kernel launches issued so far by this context (all streams, graphs counted
 * per kernel node replayed). */
swe_status swe_launch_count(swe_ctx* ctx, int64_t* n);
/* Blocks until the context's stream is idle and checks the device error word. */
swe_status swe_synchronize(swe_ctx* ctx);

/* Message of the last failure on ctx (NULL ctx: the last failure of a create
 * on this thread).  Never NULL. */
const char* swe_last_error(swe_ctx* ctx);

/* Simulated time accumulated by CFL runs (swe_run_cfl's t_elapsed); set it
 * when resuming from a checkpoint.  No reference counterpart (its driver
 * keeps t itself, examples/Main.cpp:237-241). */
swe_status swe_get_time(swe_ctx* ctx, double* t);
swe_status swe_set_time(swe_ctx* ctx, double t);
/* Sets the CFL ratio that the next CFL step's dt is taken from (the
 * reference's m_min_length_to_wavespeed, include/SpaceDisc.h:43): a resumed
 * run takes the ratio its checkpoint recorded, which came from the last
 * stage's flux pass, not from a pass over the final state. */
swe_status swe_set_min_len_to_wavespeed(swe_ctx* ctx, double r);

/* Time-scheme plugin: defines SWE_SCHEME_CUSTOM as a Shu-Osher table of
 * n_stages (1 to 4) stages, the form the reference's Solvers are written in
 * (src/Solvers.cpp:5-59): U_s = a[s] U0 + b[s] U_{s-1} + RHS(U_{s-1}, c[s] dt)
 * with U_{-1} = U0, each stage written through ConsAssigner; a[s] + b[s] = 1
 * and c[s] > 0.  Euler is {1}, {0}, {1}; SSPRK2 {1, 0.5}, {0, 0.5}, {1, 0.5};
 * SSPRK3 {1, 0.75, 1/3}, {0, 0.25, 2/3}, {1, 0.25, 2/3}.  Every entry point
 * that takes a scheme (steps, CFL runs, kernel timing, the adjoint) then
 * accepts SWE_SCHEME_CUSTOM; redefining it replaces the table for later calls
 * (a taped adjoint run keeps the table it ran with). */
swe_status swe_set_scheme(swe_ctx* ctx, int32_t n_stages, const double* a, const double* b, const double* c);

/* What the tuner chose: out4 = {device order (swe_reorder), threads per block
 * of the reconstruction kernels, of the edge-flux kernel, of the drain and
 * update kernels}.  Block sizes are timed at creation when swe_params.block
 * is 0 (64, 128 and 256 threads; steps run on a copy of the state, which is
 * then restored) and cached per device, flux, wave speed and log2 of the
 * cell count.  No reference counterpart (the reference has no tuner). */
swe_status swe_get_tuning(swe_ctx* ctx, int32_t* out4);

/* Host-only planning of a device order (AUTO: the cost-model choice):
 * cell_from[C], edge_from[E], node_from[N] (each optional) receive the
 * caller's index at every device position; cost3 (optional) the gathered
 * sectors of KEEP, MORTON and RCM (AUTO fills all three, a fixed strategy its
 * own); chosen the strategy used.  Needs no GPU. */
swe_status swe_layout_plan(const swe_mesh* mesh, int32_t strategy, int64_t* cell_from, int64_t* edge_from,
                           int64_t* node_from, double* cost3, int32_t* chosen);

/* Edge-flux pass that allocates no device memory, for callers that cannot call
 * cudaMalloc (a framework owning all device memory through its own pool, a
 * real-time loop that forbids allocation, a plugin handed only device
 * pointers).  No counterpart in the reference.
 *
 * For n_edges interior edges it evaluates the flux plugin (flux x wavespeed)
 * exactly as one edge of SpaceDisc::ComputeFluxes does, and the minimum
 * length-to-wavespeed ratio, reset to 1 first.  All pointers are device
 * memory: edge_geom 6 x n_edges column-major (nx, ny, tx, ty, b, lmin per edge:
 * the owner's outward normal and tangent, edge-centre bathymetry and
 * min(2 A_owner / L, 2 A_neighbour / L)); left / right 3 x n_edges interface
 * primitives (w, u, v) of the owner and the neighbour; flux_out 3 x n_edges;
 * ratio_out one double.  Asynchronous on `stream` (NULL = legacy default).
 *
 * Scratch lives in a static 512 KB device array held by every GPU that loads
 * this library, so n_edges is limited to 16,777,216 (larger requests return
 * SWE_ERR_INVALID_ARGUMENT).  Every call looks up that array's address in the
 * calling thread's current context (so a context switch or a device reset
 * leaves no stale address); the first call in a context also loads the
 * library's device code there, so make it before any stream capture.  All
 * calls share the array: calls that overlap on the GPU (other streams, other
 * threads) race.  An error already pending on the thread is returned as
 * SWE_ERR_CUDA before anything is launched and is left pending; otherwise
 * SWE_ERR_CUDA reports a failure of this call's own launches. */
swe_status swe_edge_fluxes_noalloc(int32_t flux, int32_t wavespeed, int64_t n_edges, const double* edge_geom,
                                   const double* left, const double* right, double cor, double* flux_out,
                                   double* ratio_out, void* stream);

/* ---------------------------------------------------------- discrete adjoint
 * No counterpart in the reference.  A taped forward run followed by its exact
 * reverse gives gradients of any function of gauge traces with respect to the
 * initial primitive state and the node bathymetry.
 *
 * swe_adjoint_forward: n_steps steps of `scheme` from the current state with
 * dt = CFLdt() before every step (recorded; the gradient treats it as fixed),
 * state checkpoints every `checkpoint_every` steps (bounded memory), and the
 * surface level w at the n_gauges cells `gauge_cells` after every
 * `obs_every`-th step written to traces_out (n_steps / obs_every rows of
 * n_gauges).  Leaves the context at the final state.
 *
 * swe_adjoint_backward: given trace_grads (same shape as the traces: the
 * derivative of the caller's loss with respect to each trace value), returns
 * grad_prim0 (3 x C, the initial (w, u, v)) and grad_bathymetry (N, the node
 * z of the geometry).  Segments are recomputed from their checkpoint with the
 * recorded dts; the reverse of each stage follows the branches the forward
 * took (limiter, dry clamps, min/max selections); roots of the partially-wet
 * reconstruction are differentiated by the implicit-function theorem. */
swe_status swe_adjoint_forward(swe_ctx* ctx, int32_t scheme, int64_t n_steps, int64_t checkpoint_every,
                               int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every, double* traces_out);
swe_status swe_adjoint_backward(swe_ctx* ctx, const double* trace_grads, double* grad_prim0, double* grad_bathymetry);
/* The n_steps dts recorded by the last swe_adjoint_forward. */
swe_status swe_adjoint_dts(swe_ctx* ctx, double* dts_out);
/* Wetting-front regularisation of the reverse (no reference counterpart).
 * Where a PartWet2 cell's node maximum comes from a partially-wet neighbour's
 * PartWet1 level b23 + cbrt(3 h K), that level's slope in w grows like
 * h^(-2/3) as the depth h -> 0; fed back through PartWet2 over many steps the
 * exact reverse then grows without bound on beds whose bumps emerge (1e129
 * after 500 steps of 64 such instances) while the forward stays smooth at
 * finite perturbations.  Below `depth` the slope is taken at h = depth
 * (scaled by (h / depth)^(2/3)).  Default 1e-3, the reference's
 * desingularisation depth (include/Assigners.h:30); 0 gives the exact derivative
 * of the discrete forward.  Takes effect at the next backward. */
swe_status swe_adjoint_set_regularisation(swe_ctx* ctx, double depth);
/* Builds the adjoint's one-time tables and work arrays (the cells around each
 * node, the twin slots of each edge, the plane-point adjoints of every cell;
 * built from the bed, so swe_set_bathymetry drops them) ahead of the first
 * taped run, which otherwise builds them itself.  No reference counterpart. */
swe_status swe_adjoint_prepare(swe_ctx* ctx);
/* swe_adjoint_forward / swe_adjoint_backward with every array in device memory
 * (gauge_cells stays on the host): traces_out, trace_grads, grad_prim0 (3 x C
 * interleaved, the caller's cell order) and grad_bathymetry (N, the caller's
 * node order) are device pointers; the work runs on the context's stream. */
swe_status swe_adjoint_forward_device(swe_ctx* ctx, int32_t scheme, int64_t n_steps, int64_t checkpoint_every,
                                      int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every,
                                      double* traces_out);
swe_status swe_adjoint_backward_device(swe_ctx* ctx, const double* trace_grads, double* grad_prim0,
                                       double* grad_bathymetry);
/* A forward run with prescribed dts and no tape: n_steps steps of `scheme`,
 * step n with dt = dts[n], and w at the gauge cells after every obs_every-th
 * step into traces_out (host, n_steps / obs_every rows of n_gauges).  With the
 * dts a taped run recorded (swe_adjoint_dts) it repeats that run's steps for a
 * perturbed initial state or bed: what finite-difference checks of the
 * adjoint need.  No reference counterpart. */
swe_status swe_run_traces(swe_ctx* ctx, int32_t scheme, int64_t n_steps, const double* dts, int32_t n_gauges,
                          const int64_t* gauge_cells, int64_t obs_every, double* traces_out);
/* Replaces the node bathymetry (N values, the caller's node order, host) of a
 * context: every mesh record that depends on it is recomputed with the
 * reference's operation order and re-uploaded in place (device order, tuning
 * and captured graphs kept); the state is kept and the adjoint's tape is
 * dropped.  The reference's geometry is a caller array (include/Bathymetry.h:
 * 42-43), so writing its z row and stepping again is the reference-side
 * equivalent.  Call swe_prime afterwards for a CFLdt() of the new bed. */
swe_status swe_set_bathymetry(swe_ctx* ctx, const double* z);
/* Recomputes the flux pass of the current state (SpaceDisc::
 * ComputeInterfaceValues + ComputeFluxes, src/SpaceDisc.cpp:33-74) so that
 * CFLdt() and the next CFL step follow from it, as after swe_create. */
swe_status swe_prime(swe_ctx* ctx);

/* ---------------------------------------------------------------- batched */
/* Many independent instances (each its own mesh, state, parameters and CFL
 * step) stepped together: cells and edges of all instances are concatenated
 * and every stage kernel covers them all in one launch.  params may be one
 * struct (n_params = 1) or one per instance. */
swe_status swe_batch_create(int32_t n_instances, const swe_mesh* meshes, const double* const* prim0,
                            const swe_params* params, int32_t n_params, swe_batch** out);
swe_status swe_batch_destroy(swe_batch* b);
/* Runs the batch's kernels on `stream` (NULL = the batch's own stream), with
 * the ordering of swe_set_stream. */
swe_status swe_batch_set_stream(swe_batch* b, void* stream);
/* n_steps steps of every instance, each with its own dt = cfl * ratio taken
 * before every step; one CUDA graph per step replayed n_steps times. */
swe_status swe_batch_run_cfl(swe_batch* b, int32_t scheme, int64_t n_steps);
/* n_steps fixed-dt steps (same dt for every instance). */
swe_status swe_batch_run(swe_batch* b, int32_t scheme, double dt, int64_t n_steps);
swe_status swe_batch_get_prim(swe_batch* b, int32_t instance, double* prim_out);
/* Sum of the dts taken by an instance so far. */
swe_status swe_batch_time(swe_batch* b, int32_t instance, double* t);
swe_status swe_batch_launch_count(swe_batch* b, int64_t* n);
/* Resume support for instance q of a batch: its time, its state (3 x C_q)
 * and its CFL ratio. */
swe_status swe_batch_set_time(swe_batch* b, int32_t q, double t);
swe_status swe_batch_set_prim(swe_batch* b, int32_t q, const double* prim_in);
swe_status swe_batch_min_len_to_wavespeed(swe_batch* b, int32_t q, double* r);
swe_status swe_batch_set_min_len_to_wavespeed(swe_batch* b, int32_t q, double r);
/* swe_set_scheme for every instance of a batch. */
swe_status swe_batch_set_scheme(swe_batch* bt, int32_t n_stages, const double* a, const double* b, const double* c);
/* swe_get_tuning for instance q of a batch (block sizes are shared). */
swe_status swe_batch_get_tuning(swe_batch* b, int32_t q, int32_t* out4);
swe_status swe_batch_synchronize(swe_batch* b);
const char* swe_batch_last_error(swe_batch* b);

/* Volume, kinetic and potential energy of the current state:
 * out3 = sum over wet cells of A (h, h (u^2 + v^2) / 2, h^2 / 2 + h b) with b
 * the centroid bathymetry (the reference's ComputeIntegrals,
 * src/SpaceDisc.cpp:76-104, commented out there; partially-wet cells use their
 * cell average).  Deterministic.  Synchronises the context's stream. */
swe_status swe_integrals(swe_ctx* ctx, double* out3);
swe_status swe_batch_integrals(swe_batch* b, int32_t instance, double* out3);

/* The discrete adjoint of a batch: as swe_adjoint_forward / _backward / _dts,
 * over all instances at once.  Cells, nodes and gauges are numbered over the
 * concatenation of the instances in creation order (instance q's cell i is
 * cell i + the cell counts of instances 0..q-1; nodes likewise); each instance
 * keeps its own CFL dt, recorded per step (dts_out is n_steps x n_instances).
 * grad_prim0 is 3 x C_total and grad_bathymetry N_total.  No reference
 * counterpart. */
swe_status swe_batch_adjoint_forward(swe_batch* b, int32_t scheme, int64_t n_steps, int64_t checkpoint_every,
                                     int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every,
                                     double* traces_out);
swe_status swe_batch_adjoint_backward(swe_batch* b, const double* trace_grads, double* grad_prim0,
                                      double* grad_bathymetry);
swe_status swe_batch_adjoint_dts(swe_batch* b, double* dts_out);
/* swe_adjoint_prepare for a batch. */
swe_status swe_batch_adjoint_prepare(swe_batch* b);
/* swe_adjoint_set_regularisation for a batch. */
swe_status swe_batch_adjoint_set_regularisation(swe_batch* b, double depth);
/* Device-memory forms of the batch adjoint, as for a single context. */
swe_status swe_batch_adjoint_forward_device(swe_batch* b, int32_t scheme, int64_t n_steps, int64_t checkpoint_every,
                                            int32_t n_gauges, const int64_t* gauge_cells, int64_t obs_every,
                                            double* traces_out);
swe_status swe_batch_adjoint_backward_device(swe_batch* b, const double* trace_grads, double* grad_prim0,
                                             double* grad_bathymetry);
/* swe_run_traces for a batch: dts is n_steps x n_instances (step-major, each
 * instance its own dt); gauges numbered over the concatenation. */
swe_status swe_batch_run_traces(swe_batch* b, int32_t scheme, int64_t n_steps, const double* dts, int32_t n_gauges,
                                const int64_t* gauge_cells, int64_t obs_every, double* traces_out);
/* swe_set_bathymetry for a batch: z[q] (N_q values, host) for every instance
 * whose bed changes, NULL for the others; one recompute and re-upload. */
swe_status swe_batch_set_bathymetry(swe_batch* b, const double* const* z);
/* swe_prime for every instance of a batch. */
swe_status swe_batch_prime(swe_batch* b);
/* swe_set_prim_device for instance q of a batch (3 x C_q interleaved, device). */
swe_status swe_batch_set_prim_device(swe_batch* b, int32_t q, const double* prim_in);

#ifdef __cplusplus
}
#endif

#endif /* SWE_FVM_GB300_H */
