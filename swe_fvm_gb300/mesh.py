"""Triangular meshes in the reference's array layout.

A mesh is held exactly as the reference's ``Topology`` + ``Domain`` take it
(include/TriangMesh.h:14-65, include/Bathymetry.h:12-49):

* ``geometry``        float64 (N, 3): node x, y and bathymetry z (the reference
  stores this as a column-major 3 x N ``Storage<3>``; a C-contiguous (N, 3)
  array has the same bytes),
* ``edge_nodes``      int64 (E, 2): the two nodes of each edge,
* ``edge_cells``      int64 (E, 2): owner cell, then the neighbour or -1 for a
  solid wall (``Boundaries::SOLID_WALL``, include/Includes.h:21),
* ``cell_nodes``      int64 (C, 3),
* ``cell_edges``      int64 (C, 3): edge k joins cell nodes k and k+1,
* ``cell_neighbours`` int64 (C, 3): neighbour k lies across edge k, -1 at a wall.

These conventions were checked on the reference's own dump
(notebooks/topology.dat, written by examples/Main.cpp:146-165).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Mesh:
    geometry: np.ndarray
    edge_nodes: np.ndarray
    edge_cells: np.ndarray
    cell_nodes: np.ndarray
    cell_edges: np.ndarray
    cell_neighbours: np.ndarray

    @property
    def num_nodes(self) -> int:
        return int(self.geometry.shape[0])

    @property
    def num_edges(self) -> int:
        return int(self.edge_nodes.shape[0])

    @property
    def num_cells(self) -> int:
        return int(self.cell_nodes.shape[0])

    def centroids(self) -> np.ndarray:
        """Cell centroids as Domain::T computes them (src/Bathymetry.cpp:24-27)."""
        g = self.geometry
        k = 1.0 / 3.0
        p = g[self.cell_nodes]  # (C, 3, 3)
        return p[:, 0] * k + p[:, 1] * k + p[:, 2] * k

    def areas(self) -> np.ndarray:
        g = self.geometry
        p = g[self.cell_nodes]
        ba = p[:, 1, :2] - p[:, 0, :2]
        ca = p[:, 2, :2] - p[:, 0, :2]
        return 0.5 * np.abs(ba[:, 0] * ca[:, 1] - ca[:, 0] * ba[:, 1])

    def contiguous(self) -> "Mesh":
        return Mesh(
            np.ascontiguousarray(self.geometry, dtype=np.float64),
            np.ascontiguousarray(self.edge_nodes, dtype=np.int64),
            np.ascontiguousarray(self.edge_cells, dtype=np.int64),
            np.ascontiguousarray(self.cell_nodes, dtype=np.int64),
            np.ascontiguousarray(self.cell_edges, dtype=np.int64),
            np.ascontiguousarray(self.cell_neighbours, dtype=np.int64),
        )


def build_topology(points_xyz: np.ndarray, triangles: np.ndarray) -> Mesh:
    """Reference topology arrays from a node list and a triangle list.

    Edges are numbered in order of first appearance while walking the cells in
    order, so an edge's owner (``edge_cells[:, 0]``) is the first cell that
    touches it and edges stay local when the cells are.
    """
    tri = np.ascontiguousarray(triangles, dtype=np.int64)
    C = tri.shape[0]
    N = points_xyz.shape[0]
    a = tri
    b = np.roll(tri, -1, axis=1)  # edge k joins node k and node k+1
    lo = np.minimum(a, b).reshape(-1)
    hi = np.maximum(a, b).reshape(-1)
    key = lo * N + hi
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")  # edges by first appearance
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    eid = rank[inv]  # (3C,) edge id of each (cell, k)
    E = uniq.size
    first_sorted = first[order]
    edge_nodes = np.stack([a.reshape(-1)[first_sorted], b.reshape(-1)[first_sorted]], axis=1)
    cell_of = np.repeat(np.arange(C, dtype=np.int64), 3)
    edge_cells = np.full((E, 2), -1, dtype=np.int64)
    edge_cells[:, 0] = cell_of[first_sorted]
    # the second touching cell of each edge
    owner = edge_cells[eid, 0]
    other = cell_of != owner
    cnt = np.bincount(eid, minlength=E)
    if np.any(cnt > 2):
        raise ValueError("non-manifold mesh: an edge is shared by more than two cells")
    edge_cells[eid[other], 1] = cell_of[other]
    cell_edges = eid.reshape(C, 3)
    ec = edge_cells[cell_edges]  # (C, 3, 2)
    me = np.arange(C, dtype=np.int64)[:, None]
    nb = np.where(ec[:, :, 0] == me, ec[:, :, 1], ec[:, :, 0])
    return Mesh(
        np.ascontiguousarray(points_xyz, dtype=np.float64),
        edge_nodes.astype(np.int64),
        edge_cells,
        tri,
        cell_edges.astype(np.int64),
        nb.astype(np.int64),
    )


def _part1by1(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint64) & np.uint64(0xFFFF)
    v = (v | (v << np.uint64(8))) & np.uint64(0x00FF00FF)
    v = (v | (v << np.uint64(4))) & np.uint64(0x0F0F0F0F)
    v = (v | (v << np.uint64(2))) & np.uint64(0x33333333)
    v = (v | (v << np.uint64(1))) & np.uint64(0x55555555)
    return v


def morton_order(xy: np.ndarray) -> np.ndarray:
    """Permutation that sorts 2-D points along a 16-bit-per-axis Z curve."""
    lo = xy.min(axis=0)
    span = np.maximum(xy.max(axis=0) - lo, 1e-300)
    q = np.clip(((xy - lo) / span * 65535.0).astype(np.int64), 0, 65535)
    code = _part1by1(q[:, 0]) | (_part1by1(q[:, 1]) << np.uint64(1))
    return np.argsort(code, kind="stable")


def reorder_morton(points_xyz: np.ndarray, triangles: np.ndarray):
    """Morton order of cells (by centroid) and of nodes (by position)."""
    node_perm = morton_order(points_xyz[:, :2])
    inv = np.empty_like(node_perm)
    inv[node_perm] = np.arange(node_perm.size)
    pts = points_xyz[node_perm]
    tri = inv[triangles]
    cen = pts[tri][:, :, :2].mean(axis=1)
    cell_perm = morton_order(cen)
    return pts, tri[cell_perm]


def renumbered(m: Mesh, cell_from, edge_from, node_from) -> Mesh:
    """The same mesh with cells, edges and nodes renumbered: new cell j is old
    cell cell_from[j] (likewise edges and nodes); every cell's and edge's own
    row order is kept, so the step computes the same values per cell."""
    cf, ef, nf = (np.asarray(a, dtype=np.int64) for a in (cell_from, edge_from, node_from))
    ic, ie, inn = np.empty_like(cf), np.empty_like(ef), np.empty_like(nf)
    ic[cf], ie[ef], inn[nf] = np.arange(cf.size), np.arange(ef.size), np.arange(nf.size)

    def cells(a):
        return np.where(a >= 0, ic[np.maximum(a, 0)], a)

    return Mesh(m.geometry[nf].copy(), inn[m.edge_nodes[ef]], cells(m.edge_cells[ef]), inn[m.cell_nodes[cf]],
                ie[m.cell_edges[cf]], cells(m.cell_neighbours[cf])).contiguous()


def shuffled(m: Mesh, seed: int):
    """m with cells, edges and nodes numbered at random (a worst case for
    memory locality).  Returns (mesh, cell_from, edge_from, node_from)."""
    rng = np.random.default_rng(seed)
    cf, ef, nf = rng.permutation(m.num_cells), rng.permutation(m.num_edges), rng.permutation(m.num_nodes)
    return renumbered(m, cf, ef, nf), cf, ef, nf


def structured_square(n: int, lo: float, hi: float, bathymetry=None) -> Mesh:
    """[lo, hi]^2 split into n x n squares, 2 triangles each.

    Each square (i, j) with corners a=(i,j), b=(i+1,j), c=(i+1,j+1), d=(i,j+1)
    is cut along its a-c diagonal into (a, b, c) and (a, c, d).
    """
    xs = np.linspace(lo, hi, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    pts = np.zeros(((n + 1) * (n + 1), 3))
    pts[:, 0] = X.reshape(-1)
    pts[:, 1] = Y.reshape(-1)
    if bathymetry is not None:
        pts[:, 2] = bathymetry(pts[:, 0], pts[:, 1])
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = (j * (n + 1) + i).reshape(-1)
    b = a + 1
    c = a + (n + 1) + 1
    d = a + (n + 1)
    t1 = np.stack([a, b, c], axis=1)
    t2 = np.stack([a, c, d], axis=1)
    tri = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return build_topology(pts, tri)


def jittered_delaunay(m: int, seed: int, jitter: float = 0.3, morton: bool = True) -> tuple:
    """Delaunay triangulation of an m x m jittered lattice on the unit square.

    Interior lattice points move by U(-jitter, jitter) * spacing in x and y;
    boundary points stay on the square's sides so the hull is the square.
    Returns (points (N, 3) with z = 0, triangles (C, 3)).
    """
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 1.0, m)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    pts = np.stack([X.reshape(-1), Y.reshape(-1)], axis=1)
    h = 1.0 / (m - 1)
    interior = (pts[:, 0] > 0) & (pts[:, 0] < 1) & (pts[:, 1] > 0) & (pts[:, 1] < 1)
    jit = rng.uniform(-jitter, jitter, size=pts.shape) * h
    pts[interior] += jit[interior]
    tri = Delaunay(pts, qhull_options="Qbb Qc Qz Q12").simplices.astype(np.int64)
    p = pts[tri]
    area2 = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    tri = tri[np.abs(area2) > 1e-6 * h * h]
    xyz = np.zeros((pts.shape[0], 3))
    xyz[:, :2] = pts
    if morton:
        xyz, tri = reorder_morton(xyz, tri)
    return xyz, tri


def gaussian_bumps(x, y, amps, widths, centres):
    b = np.zeros_like(x)
    for A, s, (cx, cy) in zip(amps, widths, centres):
        b += A * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2.0 * s * s))
    return np.maximum(b, 0.0)


def triang_average(p0, p1, p2, f, n: int):
    """Cell average of f over triangles (p0, p1, p2), vectorised over cells.

    The quadrature of ``TriangAverage<k, n>`` (include/PointOperations.h:20-44):
    f is sampled at the centroids of the n^2 congruent sub-triangles, each with
    weight 1/n^2.  f maps (x, y) arrays of shape (C, S) to an array (k, C, S).
    """
    h = 1.0 / n
    di = h * (p1 - p0)
    dj = h * (p2 - p0)
    dt = (di + dj) / 3.0
    ii, jj = [], []
    up_i, up_j, dn_i, dn_j = [], [], [], []
    for i in range(n):
        for j in range(n - i):
            up_i.append(i)
            up_j.append(j)
        for j in range(n - i - 1):
            dn_i.append(i)
            dn_j.append(j)
    up_i = np.array(up_i, dtype=np.float64)
    up_j = np.array(up_j, dtype=np.float64)
    dn_i = np.array(dn_i, dtype=np.float64)
    dn_j = np.array(dn_j, dtype=np.float64)
    ii = np.concatenate([up_i, dn_i])
    jj = np.concatenate([up_j, dn_j])
    shift = np.concatenate([np.ones_like(up_i), 2.0 * np.ones_like(dn_i)])
    x = p0[:, None, 0] + ii[None, :] * di[:, None, 0] + jj[None, :] * dj[:, None, 0] + shift[None, :] * dt[:, None, 0]
    y = p0[:, None, 1] + ii[None, :] * di[:, None, 1] + jj[None, :] * dj[:, None, 1] + shift[None, :] * dt[:, None, 1]
    vals = f(x, y)
    return vals.mean(axis=-1)


def load_reference_dump(geometry_path: str, topology_path: str) -> Mesh:
    """Read the text dump written by examples/Main.cpp:126-170 (dumpDomain)."""
    geo = np.loadtxt(geometry_path, dtype=np.float64).reshape(-1, 3)
    with open(topology_path) as fh:
        lines = fh.read().split("\n")
    E = int(lines[0])
    ed = np.array([[int(v) for v in lines[1 + e].split()] for e in range(E)], dtype=np.int64)
    C = int(lines[1 + E])
    cd = np.array([[int(v) for v in lines[2 + E + c].split()] for c in range(C)], dtype=np.int64)
    return Mesh(geo, ed[:, :2].copy(), ed[:, 2:].copy(), cd[:, :3].copy(), cd[:, 3:6].copy(), cd[:, 6:].copy())
