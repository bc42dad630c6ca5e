"""Seeded synthetic workloads (mesh + initial primitive state).

Each builder returns ``(mesh, prim0)`` with ``prim0`` float64 (C, 3) holding
(w, u, v) per cell: free-surface level and velocity, the reference's volume
field layout (include/ValueField.h:31-48; a column-major 3 x C array has the
same bytes).

* ``thacker``        -- classic Thacker parabolic bowl on a structured square
  mesh (examples/Tests.h:237-280 with cor = 0), cell-averaged like
  examples/Main.cpp:207-223.
* ``dam_break``      -- jittered-lattice Delaunay mesh of the unit square with
  Gaussian bumps and a dam-break step over them (wet/dry fronts).
* ``hump_instance``  -- one member of the ensemble: still water of depth 0.1
  over 1-4 bumps plus a Gaussian hump of surface elevation.
* ``lake_at_rest``   -- still water over a stepped bowl (examples/Tests.h:32-43).
* ``gauss_wave``     -- the reference driver's Gaussian hump
  (examples/Main.cpp:172-195).
"""
from __future__ import annotations

import math

import numpy as np

from .mesh import Mesh, build_topology, gaussian_bumps, jittered_delaunay, structured_square, triang_average


def _cell_b(mesh: Mesh) -> np.ndarray:
    return mesh.centroids()[:, 2]


# --------------------------------------------------------------------- Thacker
class ClassicThacker:
    """Closed-form parabolic-bowl solution, examples/Tests.h:135-162, 237-280.

    Bowl ``b = delta * (x^2 + y^2)`` (BowlTest's delta*(r^2 - 1) shifted by
    +delta; only depth matters), centre at the origin, no Coriolis.
    """

    def __init__(self, delta=0.1, H0=math.sqrt(0.3), p0=0.0, q0=0.0, cor=0.0):
        self.delta, self.H0, self.p0, self.q0, self.cor = delta, H0, p0, q0, cor
        self.w = math.sqrt(cor * cor + 8.0 * delta)
        qz = (q0 - 0.5 * cor) ** 2
        rz = qz + 2.0 * H0 * H0 + p0 * p0 - 0.25 * self.w * self.w
        self.a = math.sqrt(rz * rz + self.w * self.w * p0 * p0) / (rz + 0.5 * self.w * self.w)
        self.b = math.atan(self.w * p0 / rz)

    def _den(self, t):
        return 1.0 - self.a * math.cos(self.w * t + self.b)

    def p(self, t):
        return 0.5 * self.w * self.a * math.sin(self.w * t + self.b) / self._den(t)

    def q(self, t):
        return (self.q0 - 0.5 * self.cor) * (1.0 - self.a * math.cos(self.b)) / self._den(t) + 0.5 * self.cor

    def Hc(self, t):
        return self.H0 * (1.0 - self.a * math.cos(self.b)) / self._den(t)

    def Hxx(self, t):
        qz = (self.q0 - 0.5 * self.cor) ** 2
        az0 = (1.0 - self.a * math.cos(self.b)) ** 2
        azt = self._den(t) ** 2
        return (0.25 * self.w * self.w * (self.a * self.a - 1.0) + qz * az0) / azt

    def h(self, x, y, t):
        r = self.Hc(t) + 0.5 * self.Hxx(t) * x * x + 0.5 * self.Hxx(t) * y * y
        return np.maximum(0.0, r)

    def u(self, x, y, t):
        return self.p(t) * x + self.q(t) * y

    def v(self, x, y, t):
        return self.q(t) * (-x) + self.p(t) * y

    def bed(self, x, y):
        return self.delta * (x * x + y * y)

    def period(self):
        return 2.0 * math.pi / self.w


def thacker(n: int = 64, quad: int = 100, t: float = 0.0):
    """Workload: [-2,2]^2, n x n squares x 2 triangles (8192 cells at n=64),
    bed 0.1 (x^2+y^2), Thacker amplitude a = 0.5 (H0 = sqrt(0.3), p0 = q0 = 0)."""
    th = ClassicThacker()
    mesh = structured_square(n, -2.0, 2.0, bathymetry=th.bed)
    g = mesh.geometry
    p = g[mesh.cell_nodes]
    avg = np.zeros((mesh.num_cells, 3))
    chunk = 4096
    for s in range(0, mesh.num_cells, chunk):
        sl = slice(s, s + chunk)
        f = lambda x, y: np.stack([th.h(x, y, t), th.u(x, y, t) * np.ones_like(x), th.v(x, y, t) * np.ones_like(x)])
        avg[sl] = triang_average(p[sl, 0], p[sl, 1], p[sl, 2], f, quad).T
    prim = avg.copy()
    prim[:, 0] += _cell_b(mesh)
    return mesh, prim


# ------------------------------------------------------------------- dam break
def dam_break(lattice: int = 708, seed_mesh: int = 0, seed_bed: int = 1, n_bumps: int = 8):
    """Workload: Delaunay of a lattice x lattice jittered grid (about 2 lattice^2
    triangles; 708 -> ~1.0M), Morton order; 8 bumps with heights U[0.05,0.3],
    widths U[0.02,0.1] over a flat floor at 0; w0 = 0.5 for x < 0.3 else 0.2,
    raised to the cell bed where bumps emerge; u = v = 0."""
    xyz, tri = jittered_delaunay(lattice, seed_mesh)
    rng = np.random.default_rng(seed_bed)
    amps = rng.uniform(0.05, 0.3, n_bumps)
    widths = rng.uniform(0.02, 0.1, n_bumps)
    centres = rng.uniform(0.0, 1.0, (n_bumps, 2))
    xyz[:, 2] = gaussian_bumps(xyz[:, 0], xyz[:, 1], amps, widths, centres)
    mesh = build_topology(xyz, tri)
    cen = mesh.centroids()
    w0 = np.where(cen[:, 0] < 0.3, 0.5, 0.2)
    w0 = np.maximum(w0, cen[:, 2])
    prim = np.zeros((mesh.num_cells, 3))
    prim[:, 0] = w0
    return mesh, prim


def hump_instance(seed: int, cells: int):
    """Ensemble member: seeded Delaunay mesh with about `cells` triangles,
    1-4 bumps, still water at depth 0.1 plus a Gaussian surface hump with
    amplitude U[0.01,0.2] and width U[0.05,0.2]."""
    rng = np.random.default_rng(seed)
    lattice = max(8, int(round(math.sqrt(cells / 2.0))) + 1)
    xyz, tri = jittered_delaunay(lattice, seed)
    nb = int(rng.integers(1, 5))
    amps = rng.uniform(0.05, 0.3, nb)
    widths = rng.uniform(0.02, 0.1, nb)
    centres = rng.uniform(0.0, 1.0, (nb, 2))
    xyz[:, 2] = gaussian_bumps(xyz[:, 0], xyz[:, 1], amps, widths, centres)
    mesh = build_topology(xyz, tri)
    cen = mesh.centroids()
    A = rng.uniform(0.01, 0.2)
    s = rng.uniform(0.05, 0.2)
    c = rng.uniform(0.2, 0.8, 2)
    w0 = 0.1 + A * np.exp(-((cen[:, 0] - c[0]) ** 2 + (cen[:, 1] - c[1]) ** 2) / (2 * s * s))
    prim = np.zeros((mesh.num_cells, 3))
    prim[:, 0] = np.maximum(w0, cen[:, 2])
    return mesh, prim


def sloped_bump_case(lattice: int = 25, seed: int = 9):
    """Jittered-lattice Delaunay mesh of the unit square over a bed that is
    sloped everywhere (a tilt plus one broad bump that emerges), a Gaussian
    hump and a background current: no flat regions, so the binary limiter and
    the HLLC star-velocity switch are away from their kinks except at the
    wet/dry front (used by the adjoint's finite-difference checks)."""
    xyz, tri = jittered_delaunay(lattice, seed)
    x, y = xyz[:, 0], xyz[:, 1]
    xyz[:, 2] = 0.08 * x + 0.05 * y + 0.25 * np.exp(-((x - 0.7) ** 2 + (y - 0.35) ** 2) / (2 * 0.12 ** 2))
    mesh = build_topology(xyz, tri)
    cen = mesh.centroids()
    w0 = 0.2 + 0.04 * np.exp(-((cen[:, 0] - 0.3) ** 2 + (cen[:, 1] - 0.6) ** 2) / (2 * 0.1 ** 2))
    prim = np.zeros((mesh.num_cells, 3))
    prim[:, 0] = np.maximum(w0, cen[:, 2])
    wet = prim[:, 0] - cen[:, 2] > 1e-12
    prim[wet, 1] = 0.05
    prim[wet, 2] = 0.03
    return mesh, prim


def ensemble_sizes(n_instances: int = 256, lo: int = 2000, hi: int = 200000, seed: int = 7):
    """Cell counts log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(math.log(lo), math.log(hi), n_instances)).astype(np.int64)


def _hump_job(args):
    seed, cells = args
    return hump_instance(seed, cells)


def ensemble(n_instances: int = 256, lo: int = 2000, hi: int = 200000, seed0: int = 1000, processes: int = 0):
    """Workload: n_instances seeded instances (instance i uses seed seed0 + i) with
    cell counts log-uniform in [lo, hi].  Generated in `spawn` worker processes
    (safe to call before or after CUDA is initialised in the parent)."""
    import multiprocessing as mp
    import os

    sizes = ensemble_sizes(n_instances, lo, hi)
    jobs = [(seed0 + i, int(c)) for i, c in enumerate(sizes)]
    nproc = processes or max(1, min(16, (os.cpu_count() or 1)))
    if nproc == 1:
        return [_hump_job(j) for j in jobs]
    with mp.get_context("spawn").Pool(nproc) as pool:
        return pool.map(_hump_job, jobs, chunksize=1)


def adjoint_ensemble(n_instances: int = 64, lo: int = 20000, hi: int = 100000, seed0: int = 5000,
                     processes: int = 0):
    """Batched-adjoint config: n_instances seeded instances (the ensemble's
    generator, instance i with seed seed0 + i) with cell counts uniform in
    [lo, hi]."""
    import multiprocessing as mp
    import os

    sizes = np.random.default_rng(seed0).uniform(lo, hi, n_instances)
    jobs = [(seed0 + i, int(c)) for i, c in enumerate(sizes)]
    nproc = processes or max(1, min(16, (os.cpu_count() or 1)))
    if nproc == 1:
        return [_hump_job(j) for j in jobs]
    with mp.get_context("spawn").Pool(nproc) as pool:
        return pool.map(_hump_job, jobs, chunksize=1)


# ---------------------------------------------------------------- small cases
def lake_at_rest(n: int = 32, level: float = 0.0):
    """Still water over a stepped bed on [0,4]^2 (examples/Tests.h:37-42): bed
    -0.2 inside (1,3)^2 and -1 elsewhere at the nodes; w = max(level, b_cell)."""
    def bed(x, y):
        return np.where((1 < x) & (x < 3) & (1 < y) & (y < 3), -0.2, -1.0)

    mesh = structured_square(n, 0.0, 4.0, bathymetry=bed)
    prim = np.zeros((mesh.num_cells, 3))
    prim[:, 0] = np.maximum(level, _cell_b(mesh))
    return mesh, prim


def gauss_wave(mesh: Mesh, centre=(4.0, 4.0)):
    """w = 1 + exp(-5 r^2) about `centre` at the cell centroids, flat bed
    (examples/Main.cpp:182-186)."""
    cen = mesh.centroids()
    r = (cen[:, 0] - centre[0]) ** 2 + (cen[:, 1] - centre[1]) ** 2
    prim = np.zeros((mesh.num_cells, 3))
    prim[:, 0] = 1.0 + np.exp(-5.0 * r)
    return prim


def random_front_case(n: int = 24, seed: int = 0):
    """Small mesh with every reconstruction branch: bumps that emerge through
    the surface, dry islands, thin films and a velocity field."""
    rng = np.random.default_rng(seed)
    xyz, tri = jittered_delaunay(n, seed)
    nb = 5
    xyz[:, 2] = gaussian_bumps(xyz[:, 0], xyz[:, 1], rng.uniform(0.1, 0.4, nb), rng.uniform(0.05, 0.15, nb),
                               rng.uniform(0.1, 0.9, (nb, 2)))
    mesh = build_topology(xyz, tri)
    cen = mesh.centroids()
    w0 = 0.15 + 0.1 * np.exp(-((cen[:, 0] - 0.3) ** 2 + (cen[:, 1] - 0.6) ** 2) / 0.02)
    w0 = np.maximum(w0, cen[:, 2])
    # thin films on a few cells
    thin = rng.random(mesh.num_cells) < 0.05
    w0[thin] = cen[thin, 2] + rng.uniform(0.0, 2e-3, thin.sum())
    prim = np.zeros((mesh.num_cells, 3))
    prim[:, 0] = w0
    wet = w0 - cen[:, 2] > 1e-12
    prim[wet, 1] = rng.normal(0, 0.2, wet.sum())
    prim[wet, 2] = rng.normal(0, 0.2, wet.sum())
    return mesh, prim
