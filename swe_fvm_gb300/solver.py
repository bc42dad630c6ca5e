"""Host-side mirror of the reference's solver API over the GPU library.

Names, argument meaning and error behaviour follow NikitaMatckevich/SWE_FVM:

* ``Topology.create(numNodes, edgeNodes, edgeElements, elementNodes,
  elementEdges, elementNeighbours)`` -- pybind/Topology.cpp:8-31 (the arrays are
  copied; the reference's binding keeps dangling references to them),
* ``Domain(geometry, topology)`` -- src/Bathymetry.cpp:6-8,
* ``Fluxes.HLL(Wavespeeds.X)`` / ``Fluxes.HLLC(Wavespeeds.X)`` -- the flux
  plugins of include/Fluxes.h:14-111 over the wave speeds of src/Fluxes.cpp:5-26,
* ``SpaceDisc(fluxer, domain, v0, cor=0, tau=0)`` -- include/SpaceDisc.h:20-48,
* ``TimeDisc(sd)`` with ``CFLdt()`` -- include/TimeDisc.h:4-23,
* ``Solvers.Euler / SSPRK2 / SSPRK3(td, dt)`` -- include/Solvers.h:4-10, and
  ``Solvers.Custom`` for a caller's Shu-Osher table (``SpaceDisc.set_scheme``).

Beyond the reference: ``Batch`` (many meshes per launch), the device order and
block-size tuner (``reorder=``, ``block=``, ``tuning()``, ``layout_plan``),
checkpoints (``save`` / ``restore``) and device-pointer state I/O.

The reference raises DomainError / SolverError (include/Exceptions.h:4-10);
here every failure is a ``SweError`` (a RuntimeError) carrying the library's
status code and message.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import SweError, SweMesh, SweParams, check
from .mesh import Mesh


def _i64(a, shape):
    a = np.ascontiguousarray(a, dtype=np.int64)
    if a.ndim != 2 or a.shape[1] != shape:
        raise ValueError(f"expected an (n, {shape}) int64 array, got shape {a.shape}")
    return a


class Topology:
    """Connectivity arrays of a triangular mesh (include/TriangMesh.h:14-65)."""

    def __init__(self, numNodes, edgeNodes, edgeElements, elementNodes, elementEdges, elementNeighbours):
        self._n = int(numNodes)
        self.edge_nodes = _i64(edgeNodes, 2)
        self.edge_cells = _i64(edgeElements, 2)
        self.cell_nodes = _i64(elementNodes, 3)
        self.cell_edges = _i64(elementEdges, 3)
        self.cell_neighbours = _i64(elementNeighbours, 3)

    @staticmethod
    def create(numNodes, edgeNodes, edgeElements, elementNodes, elementEdges, elementNeighbours) -> "Topology":
        return Topology(numNodes, edgeNodes, edgeElements, elementNodes, elementEdges, elementNeighbours)

    def num_nodes(self) -> int:
        return self._n

    def num_edges(self) -> int:
        return int(self.edge_nodes.shape[0])

    def num_elements(self) -> int:
        return int(self.cell_nodes.shape[0])

    def IsEdgeBoundary(self, e: int) -> bool:  # src/TriangMesh.cpp:5-7
        return bool(self.edge_cells[e, 1] < 0)

    def IsTriangleBoundary(self, t: int) -> bool:  # src/TriangMesh.cpp:18-23
        return bool(np.any(self.edge_cells[self.cell_edges[t], 1] < 0))


class Domain:
    """Geometry (x, y, bathymetry z per node) over a Topology."""

    def __init__(self, geometry, topology: Topology):
        g = np.ascontiguousarray(geometry, dtype=np.float64)
        if g.ndim == 2 and g.shape[0] == 3 and g.shape[1] != 3:
            g = np.ascontiguousarray(g.T)  # a 3 x N array as the reference stores it
        if g.shape != (topology.num_nodes(), 3):
            raise ValueError(f"geometry must be (num_nodes, 3) or (3, num_nodes); got {g.shape}")
        self.geometry = g
        self.topology = topology

    @staticmethod
    def from_mesh(m: Mesh) -> "Domain":
        t = Topology(m.num_nodes, m.edge_nodes, m.edge_cells, m.cell_nodes, m.cell_edges, m.cell_neighbours)
        return Domain(m.geometry, t)

    def mesh(self) -> Mesh:
        t = self.topology
        return Mesh(self.geometry, t.edge_nodes, t.edge_cells, t.cell_nodes, t.cell_edges, t.cell_neighbours)

    def GetTopology(self) -> Topology:
        return self.topology


class Wavespeeds:
    """Wave-speed plugins (src/Fluxes.cpp:5-26)."""

    Rusanov = 0
    Davis = 1
    Einfeldt = 2


@dataclass(frozen=True)
class Fluxer:
    kind: int  # 0 HLL, 1 HLLC
    wavespeed: int


class Fluxes:
    """Flux plugins (include/Fluxes.h:14-111)."""

    @staticmethod
    def HLL(wavespeed=Wavespeeds.Einfeldt) -> Fluxer:
        return Fluxer(0, int(wavespeed))

    @staticmethod
    def HLLC(wavespeed=Wavespeeds.Einfeldt) -> Fluxer:
        return Fluxer(1, int(wavespeed))


def _swe_mesh(m: Mesh):
    keep = m.contiguous()
    sm = SweMesh(
        keep.num_nodes, keep.num_edges, keep.num_cells,
        keep.geometry.ctypes.data, keep.edge_nodes.ctypes.data, keep.edge_cells.ctypes.data,
        keep.cell_nodes.ctypes.data, keep.cell_edges.ctypes.data, keep.cell_neighbours.ctypes.data,
    )
    return sm, keep


REORDER = {"auto": -1, "keep": 0, "morton": 1, "rcm": 2}


def make_params(fluxer: Fluxer, cor=0.0, tau=0.0, cfl=0.15, reorder="auto", block=0) -> SweParams:
    """swe_params for a flux plugin; ``reorder`` is one of REORDER's keys (the
    device order of cells, edges and nodes), ``block`` the threads per block
    (0: timed at creation)."""
    L = _lib.load()
    p = SweParams()
    L.swe_params_default(ctypes.byref(p))
    p.flux = fluxer.kind
    p.wavespeed = fluxer.wavespeed
    p.cor = float(cor)
    p.tau = float(tau)
    p.cfl = float(cfl)
    p.reorder = REORDER[reorder] if isinstance(reorder, str) else int(reorder)
    p.block = int(block)
    return p


def _tuning(out: np.ndarray) -> dict:
    names = {v: k for k, v in REORDER.items()}
    return {"reorder": names.get(int(out[0]), int(out[0])), "block_recon": int(out[1]), "block_flux": int(out[2]),
            "block_update": int(out[3])}


def layout_plan(mesh: Mesh, reorder="auto") -> dict:
    """The device order swe_create would use for ``mesh`` (host only, no GPU):
    cell_from / edge_from / node_from give the mesh's index at every device
    position, cost the gathered 32-byte sectors of keep, morton and rcm, and
    chosen the strategy."""
    L = _lib.load()
    sm, keep = _swe_mesh(mesh)
    cf = np.empty(mesh.num_cells, dtype=np.int64)
    ef = np.empty(mesh.num_edges, dtype=np.int64)
    nf = np.empty(mesh.num_nodes, dtype=np.int64)
    cost = np.zeros(3)
    chosen = ctypes.c_int32()
    code = REORDER[reorder] if isinstance(reorder, str) else int(reorder)
    st = L.swe_layout_plan(ctypes.byref(sm), code, cf.ctypes.data, ef.ctypes.data, nf.ctypes.data, cost.ctypes.data,
                           ctypes.byref(chosen))
    check(st, None)
    names = {v: k for k, v in REORDER.items()}
    return {"cell_from": cf, "edge_from": ef, "node_from": nf, "cost": cost, "chosen": names[chosen.value]}


class SpaceDisc:
    """Device-resident SpaceDisc (include/SpaceDisc.h:20-48).

    ``v0`` is the initial primitive field, (C, 3) = (w, u, v) per cell.  All
    arrays are copied to the current CUDA device.
    """

    def __init__(self, fluxer: Fluxer, domain, v0, cor: float = 0.0, tau: float = 0.0, cfl: float = 0.15,
                 reorder="auto", block: int = 0):
        L = _lib.load()
        if isinstance(domain, Mesh):
            domain = Domain.from_mesh(domain)
        self.domain = domain
        self.fluxer = fluxer
        self.cor, self.tau, self.cfl = float(cor), float(tau), float(cfl)
        m = domain.mesh()
        sm, self._keep = _swe_mesh(m)
        prim = np.ascontiguousarray(v0, dtype=np.float64).reshape(m.num_cells, 3)
        p = make_params(fluxer, cor, tau, cfl, reorder, block)
        ctx = ctypes.c_void_p()
        st = L.swe_create(ctypes.byref(sm), prim.ctypes.data, ctypes.byref(p), ctypes.byref(ctx))
        check(st, None)
        self.ctx = ctx
        self.num_cells = m.num_cells
        self.num_edges = m.num_edges
        self.num_nodes = m.num_nodes

    def __del__(self):
        ctx = getattr(self, "ctx", None)
        if ctx:
            try:
                _lib.load().swe_destroy(ctx)
            except Exception:
                pass
            self.ctx = None

    def _check(self, st):
        check(st, self.ctx)

    # --- reference getters
    def GetDomain(self):
        return self.domain

    def GetCor(self) -> float:
        return self.cor

    def GetTau(self) -> float:
        return self.tau

    def GetVolField(self) -> np.ndarray:
        out = np.empty((self.num_cells, 3))
        self._check(_lib.load().swe_get_prim(self.ctx, out.ctypes.data))
        return out

    def SetVolField(self, prim) -> None:
        a = np.ascontiguousarray(prim, dtype=np.float64).reshape(self.num_cells, 3)
        self._check(_lib.load().swe_set_prim(self.ctx, a.ctypes.data))

    def GetEdgField(self) -> np.ndarray:
        edg = np.empty((2 * self.num_edges, 3))
        self._check(_lib.load().swe_get_edge_values(self.ctx, edg.ctypes.data, None))
        return edg

    def GetSrcField(self) -> np.ndarray:
        src = np.empty((2 * self.num_edges, 3))
        self._check(_lib.load().swe_get_edge_values(self.ctx, None, src.ctypes.data))
        return src

    def GetFluxes(self) -> np.ndarray:
        f = np.empty((self.num_edges, 3))
        self._check(_lib.load().swe_get_fluxes(self.ctx, f.ctypes.data))
        return f

    def GetNodeMax(self) -> np.ndarray:
        out = np.empty(self.num_nodes)
        self._check(_lib.load().swe_get_node_max(self.ctx, out.ctypes.data))
        return out

    def GetMinLenToWavespeed(self) -> float:
        r = ctypes.c_double()
        self._check(_lib.load().swe_min_len_to_wavespeed(self.ctx, ctypes.byref(r)))
        return r.value

    # --- reference operations
    def ComputeInterfaceValues(self) -> None:
        self._check(_lib.load().swe_compute_interface_values(self.ctx))

    def ComputeFluxes(self) -> None:
        self._check(_lib.load().swe_compute_fluxes(self.ctx))

    # --- device-side loops
    def run(self, scheme: int, dt: float, n_steps: int) -> None:
        self._check(_lib.load().swe_run(self.ctx, int(scheme), float(dt), int(n_steps)))

    def run_cfl(self, scheme: int, n_steps: int) -> float:
        t = ctypes.c_double()
        self._check(_lib.load().swe_run_cfl(self.ctx, int(scheme), int(n_steps), ctypes.byref(t)))
        return t.value

    def synchronize(self) -> None:
        self._check(_lib.load().swe_synchronize(self.ctx))

    def time_kernels(self, scheme: int, reps: int) -> np.ndarray:
        """Mean ms per launch of recon1, recon2, flux, drain, update and per step."""
        out = np.zeros(6)
        self._check(_lib.load().swe_time_kernels(self.ctx, int(scheme), int(reps), out.ctypes.data))
        return out

    def integrals(self) -> np.ndarray:
        """(volume, kinetic energy, potential energy) of the current state,
        summed on the device over the wet cells."""
        out = np.zeros(3)
        self._check(_lib.load().swe_integrals(self.ctx, out.ctypes.data))
        return out

    def launch_count(self) -> int:
        n = ctypes.c_int64()
        self._check(_lib.load().swe_launch_count(self.ctx, ctypes.byref(n)))
        return n.value

    def time(self) -> float:
        """Simulated time accumulated by CFL runs."""
        t = ctypes.c_double()
        self._check(_lib.load().swe_get_time(self.ctx, ctypes.byref(t)))
        return t.value

    def set_time(self, t: float) -> None:
        self._check(_lib.load().swe_set_time(self.ctx, float(t)))

    def save(self, path: str, step: int = 0) -> None:
        """Checkpoint of the state, the time and the CFL ratio (fileio.save_state)."""
        from .fileio import save_state

        save_state(path, self.domain.mesh(), self.GetVolField(), self.time(), step, self.GetMinLenToWavespeed())

    def restore(self, path: str) -> int:
        """Resumes from a checkpoint of this mesh: state, time and CFL ratio
        (so the continued run equals the uninterrupted one bit for bit);
        returns its step count.  A checkpoint without a ratio takes the
        restored state's own flux pass."""
        from .fileio import load_state

        st = load_state(path, self.domain.mesh())
        self.SetVolField(st.prim)
        self.set_time(st.time)
        if np.isfinite(st.cfl_ratio):
            self._check(_lib.load().swe_set_min_len_to_wavespeed(self.ctx, st.cfl_ratio))
        else:
            self.ComputeInterfaceValues()
            self.ComputeFluxes()
        return st.step

    def set_scheme(self, a, b, c) -> None:
        """Defines scheme 3 (Solvers.Custom) as the Shu-Osher table (a, b, c)."""
        a, b, c = _table(a, b, c)
        self._check(_lib.load().swe_set_scheme(self.ctx, a.size, a.ctypes.data, b.ctypes.data, c.ctypes.data))

    def tuning(self) -> dict:
        """The device order and the threads per block the context runs with."""
        out = np.zeros(4, dtype=np.int32)
        self._check(_lib.load().swe_get_tuning(self.ctx, out.ctypes.data))
        return _tuning(out)

    def get_prim_device(self, ptr: int) -> None:
        self._check(_lib.load().swe_get_prim_device(self.ctx, ctypes.c_void_p(ptr)))

    def set_prim_device(self, ptr: int) -> None:
        self._check(_lib.load().swe_set_prim_device(self.ctx, ctypes.c_void_p(ptr)))

    def set_stream(self, stream_ptr: int) -> None:
        self._check(_lib.load().swe_set_stream(self.ctx, ctypes.c_void_p(stream_ptr)))

    def set_bathymetry(self, z) -> None:
        """Replaces the node bathymetry (N values, the caller's node order):
        the mesh records are recomputed and re-uploaded in place."""
        a = np.ascontiguousarray(z, dtype=np.float64).reshape(self.num_nodes)
        self._check(_lib.load().swe_set_bathymetry(self.ctx, a.ctypes.data))

    def prime(self) -> None:
        """The flux pass of the current state (CFLdt() then follows from it)."""
        self._check(_lib.load().swe_prime(self.ctx))

    def run_traces(self, scheme: int, dts, gauges, obs_every: int) -> np.ndarray:
        """len(dts) steps with the given dts; w at the gauge cells after every
        obs_every-th step, (len(dts) // obs_every, len(gauges))."""
        d = np.ascontiguousarray(dts, dtype=np.float64)
        g = np.ascontiguousarray(gauges, dtype=np.int64)
        out = np.zeros((len(d) // obs_every, len(g)))
        self._check(_lib.load().swe_run_traces(self.ctx, int(scheme), len(d), d.ctypes.data, len(g), g.ctypes.data,
                                               int(obs_every), out.ctypes.data))
        return out


class TimeDisc:
    """TimeDisc (include/TimeDisc.h:4-23) over a SpaceDisc."""

    def __init__(self, sd: SpaceDisc = None):
        self.sd = sd

    def GetSpaceDisc(self) -> SpaceDisc:
        return self.sd

    def SetSpaceDisc(self, sd: SpaceDisc) -> None:
        self.sd = sd

    def CFLdt(self) -> float:
        dt = ctypes.c_double()
        self.sd._check(_lib.load().swe_cfl_dt(self.sd.ctx, ctypes.byref(dt)))
        return dt.value


def _table(a, b, c):
    a, b, c = (np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (a, b, c))
    if not (a.size == b.size == c.size):
        raise ValueError("a, b and c need one entry per stage")
    return a, b, c


def ssprk_m2(m: int):
    """The m-stage, second-order strong-stability-preserving Runge-Kutta
    scheme in Shu-Osher form (a, b, c): m - 1 forward-Euler stages of dt/(m-1),
    then the average with the initial state; SSP coefficient m - 1."""
    if m < 2:
        raise ValueError("m >= 2")
    a = [1.0] + [0.0] * (m - 2) + [1.0 / m]
    b = [0.0] + [1.0] * (m - 2) + [(m - 1.0) / m]
    c = [1.0 / (m - 1)] * (m - 1) + [1.0 / m]
    return a, b, c


class Solvers:
    """Time schemes (include/Solvers.h:4-10): one step with a given dt.

    A new scheme plugs in as a Shu-Osher table: ``sd.set_scheme(a, b, c)``
    (stage s: a[s] U0 + b[s] U_{s-1} + RHS(U_{s-1}, c[s] dt)), then
    ``Solvers.Custom(td, dt)`` or scheme id ``Solvers.CUSTOM`` in run/run_cfl."""

    EULER, SSPRK2_ID, SSPRK3_ID, CUSTOM = 0, 1, 2, 3

    @staticmethod
    def _step(td: TimeDisc, scheme: int, dt: float):
        sd = td.GetSpaceDisc()
        sd._check(_lib.load().swe_step(sd.ctx, scheme, float(dt)))

    @staticmethod
    def Euler(td: TimeDisc, dt: float) -> None:
        Solvers._step(td, 0, dt)

    @staticmethod
    def SSPRK2(td: TimeDisc, dt: float) -> None:
        Solvers._step(td, 1, dt)

    @staticmethod
    def SSPRK3(td: TimeDisc, dt: float) -> None:
        Solvers._step(td, 2, dt)

    @staticmethod
    def Custom(td: TimeDisc, dt: float) -> None:
        """One step of the table given to SpaceDisc.set_scheme."""
        Solvers._step(td, 3, dt)


SCHEMES = {"Euler": 0, "SSPRK2": 1, "SSPRK3": 2, "Custom": 3}


class Batch:
    """Many independent instances stepped together (one launch per stage
    kernel over all instances, each with its own CFL time step)."""

    def __init__(self, meshes, prims, fluxer: Fluxer = None, cor=0.0, cfl=0.15, reorder="auto", block: int = 0):
        L = _lib.load()
        fluxer = fluxer or Fluxes.HLLC(Wavespeeds.Einfeldt)
        n = len(meshes)
        if len(prims) != n or n == 0:
            raise ValueError("need one initial state per mesh")
        arr = (SweMesh * n)()
        self._keep = []
        ptrs = (ctypes.c_void_p * n)()
        for q, (m, p) in enumerate(zip(meshes, prims)):
            sm, keep = _swe_mesh(m)
            arr[q] = sm
            pp = np.ascontiguousarray(p, dtype=np.float64).reshape(m.num_cells, 3)
            self._keep.append((keep, pp))
            ptrs[q] = pp.ctypes.data
        params = make_params(fluxer, cor, 0.0, cfl, reorder, block)
        b = ctypes.c_void_p()
        st = L.swe_batch_create(n, arr, ptrs, ctypes.byref(params), 1, ctypes.byref(b))
        check(st, None, batch=True)
        self.b = b
        self.sizes = [m.num_cells for m in meshes]

    def __del__(self):
        b = getattr(self, "b", None)
        if b:
            try:
                _lib.load().swe_batch_destroy(b)
            except Exception:
                pass
            self.b = None

    def _check(self, st):
        check(st, self.b, batch=True)

    def run_cfl(self, scheme: int, n_steps: int) -> None:
        self._check(_lib.load().swe_batch_run_cfl(self.b, int(scheme), int(n_steps)))

    def set_stream(self, stream_ptr: int) -> None:
        self._check(_lib.load().swe_batch_set_stream(self.b, ctypes.c_void_p(stream_ptr)))

    def run(self, scheme: int, dt: float, n_steps: int) -> None:
        self._check(_lib.load().swe_batch_run(self.b, int(scheme), float(dt), int(n_steps)))

    def prim(self, q: int) -> np.ndarray:
        out = np.empty((self.sizes[q], 3))
        self._check(_lib.load().swe_batch_get_prim(self.b, int(q), out.ctypes.data))
        return out

    def time(self, q: int) -> float:
        t = ctypes.c_double()
        self._check(_lib.load().swe_batch_time(self.b, int(q), ctypes.byref(t)))
        return t.value

    def integrals(self, q: int) -> np.ndarray:
        """(volume, kinetic, potential energy) of instance q."""
        out = np.zeros(3)
        self._check(_lib.load().swe_batch_integrals(self.b, int(q), out.ctypes.data))
        return out

    def synchronize(self) -> None:
        self._check(_lib.load().swe_batch_synchronize(self.b))

    def launch_count(self) -> int:
        n = ctypes.c_int64()
        self._check(_lib.load().swe_batch_launch_count(self.b, ctypes.byref(n)))
        return n.value

    def set_prim(self, q: int, prim) -> None:
        a = np.ascontiguousarray(prim, dtype=np.float64).reshape(self.sizes[q], 3)
        self._check(_lib.load().swe_batch_set_prim(self.b, int(q), a.ctypes.data))

    def set_prim_device(self, q: int, ptr: int) -> None:
        """Instance q's state from device memory (C_q x 3 interleaved)."""
        self._check(_lib.load().swe_batch_set_prim_device(self.b, int(q), ctypes.c_void_p(ptr)))

    def set_bathymetry(self, zs) -> None:
        """zs: one array of node z per instance (None keeps that instance's)."""
        keep = [None if z is None else np.ascontiguousarray(z, dtype=np.float64) for z in zs]
        ptrs = (ctypes.c_void_p * len(keep))(*[None if z is None else z.ctypes.data for z in keep])
        self._check(_lib.load().swe_batch_set_bathymetry(self.b, ptrs))

    def prime(self) -> None:
        self._check(_lib.load().swe_batch_prime(self.b))

    def run_traces(self, scheme: int, dts, gauges, obs_every: int) -> np.ndarray:
        """dts: (n_steps, n_instances); gauges numbered over the concatenated
        cells.  Returns (n_steps // obs_every, len(gauges))."""
        d = np.ascontiguousarray(dts, dtype=np.float64)
        g = np.ascontiguousarray(gauges, dtype=np.int64)
        out = np.zeros((d.shape[0] // obs_every, len(g)))
        self._check(_lib.load().swe_batch_run_traces(self.b, int(scheme), d.shape[0], d.ctypes.data, len(g),
                                                     g.ctypes.data, int(obs_every), out.ctypes.data))
        return out

    def set_time(self, q: int, t: float) -> None:
        self._check(_lib.load().swe_batch_set_time(self.b, int(q), float(t)))

    def min_len_to_wavespeed(self, q: int) -> float:
        """Instance q's CFL ratio (its next CFL dt is cfl times this)."""
        r = ctypes.c_double()
        self._check(_lib.load().swe_batch_min_len_to_wavespeed(self.b, int(q), ctypes.byref(r)))
        return r.value

    def set_min_len_to_wavespeed(self, q: int, r: float) -> None:
        self._check(_lib.load().swe_batch_set_min_len_to_wavespeed(self.b, int(q), float(r)))

    def set_scheme(self, a, b, c) -> None:
        """Defines scheme 3 for every instance as the Shu-Osher table (a, b, c)."""
        a, b, c = _table(a, b, c)
        self._check(_lib.load().swe_batch_set_scheme(self.b, a.size, a.ctypes.data, b.ctypes.data, c.ctypes.data))

    def tuning(self, q: int = 0) -> dict:
        """Device order of instance q and the batch's threads per block."""
        out = np.zeros(4, dtype=np.int32)
        self._check(_lib.load().swe_batch_get_tuning(self.b, int(q), out.ctypes.data))
        return _tuning(out)


__all__ = ["Topology", "Domain", "Wavespeeds", "Fluxes", "Fluxer", "SpaceDisc", "TimeDisc", "Solvers", "Batch",
           "SweError", "SCHEMES", "REORDER", "layout_plan", "ssprk_m2"]
