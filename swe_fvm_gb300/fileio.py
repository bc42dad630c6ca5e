"""Mesh ingestion and the reference's text outputs.

- ``read_gmsh``: ASCII Gmsh meshes (format 2.2 or 4.1) to the reference's
  topology (notebooks/mesher.py:3-69 reads them through the gmsh API; gmsh is
  not needed here).  Triangles (element type 2) become cells; node z is the
  bathymetry; every edge with one cell is a solid wall.
- ``dump_fields``: (w, hu, hv) per cell, tab-separated
  (examples/Main.cpp:65-73, dumpFields).
- ``dump_domain`` / ``load_domain``: node geometry and topology text files
  (examples/Main.cpp:126-170, dumpGeometry2 / dumpTopology / dumpDomain).
- ``save_state`` / ``load_state``: binary checkpoints (the primitive field,
  bit for bit, the simulated time and a fingerprint of the mesh), to resume a
  run; the reference has text dumps only.
"""
from __future__ import annotations

import hashlib
from typing import NamedTuple

import numpy as np

from .mesh import Mesh, build_topology, load_reference_dump

__all__ = ["read_gmsh", "dump_fields", "dump_domain", "load_domain", "save_state", "load_state",
           "mesh_fingerprint", "State"]


def _sections(text: str) -> dict:
    out, name, body = {}, None, []
    for line in text.splitlines():
        s = line.strip()
        if s.startswith("$End"):
            if name is not None:
                out[name] = body
            name, body = None, []
        elif s.startswith("$"):
            name, body = s[1:], []
        elif name is not None and s:
            body.append(s)
    return out


def _gmsh2(sec: dict):
    nodes = sec["Nodes"]
    n = int(nodes[0])
    tags = np.empty(n, dtype=np.int64)
    xyz = np.empty((n, 3))
    for k in range(n):
        f = nodes[1 + k].split()
        tags[k] = int(f[0])
        xyz[k] = [float(f[1]), float(f[2]), float(f[3])]
    els = sec["Elements"]
    tris = []
    for line in els[1:1 + int(els[0])]:
        f = [int(v) for v in line.split()]
        if f[1] == 2:  # triangle: id type ntags tags... n0 n1 n2
            tris.append(f[3 + f[2]:6 + f[2]])
    return tags, xyz, np.array(tris, dtype=np.int64).reshape(-1, 3)


def _gmsh4(sec: dict):
    nodes = sec["Nodes"]
    n_blocks = int(nodes[0].split()[0])
    tags, coords = [], []
    pos = 1
    for _ in range(n_blocks):
        dim, _tag, parametric, count = (int(v) for v in nodes[pos].split())
        pos += 1
        tags.extend(int(nodes[pos + k]) for k in range(count))
        pos += count
        for k in range(count):
            f = nodes[pos + k].split()
            coords.append([float(f[0]), float(f[1]), float(f[2])])  # parametric coordinates follow, if any
        pos += count
    els = sec["Elements"]
    n_blocks = int(els[0].split()[0])
    tris = []
    pos = 1
    for _ in range(n_blocks):
        _dim, _tag, etype, count = (int(v) for v in els[pos].split())
        pos += 1
        if etype == 2:
            for k in range(count):
                f = [int(v) for v in els[pos + k].split()]
                tris.append(f[1:4])
        pos += count
    return np.array(tags, dtype=np.int64), np.array(coords).reshape(-1, 3), np.array(tris, dtype=np.int64).reshape(-1, 3)


def read_gmsh(path: str, bathymetry=None) -> Mesh:
    """ASCII Gmsh mesh -> Mesh.  bathymetry(x, y), if given, replaces the
    node z.  Nodes not used by any triangle are dropped; the rest keep the
    file's order."""
    with open(path) as fh:
        sec = _sections(fh.read())
    if "MeshFormat" not in sec:
        raise ValueError(f"{path}: no $MeshFormat section")
    version, binary = sec["MeshFormat"][0].split()[:2]
    if binary != "0":
        raise ValueError(f"{path}: binary Gmsh files are not supported")
    if version.startswith("2"):
        tags, xyz, tris = _gmsh2(sec)
    elif version.startswith("4"):
        tags, xyz, tris = _gmsh4(sec)
    else:
        raise ValueError(f"{path}: Gmsh format {version} is not supported (2.2 or 4.1)")
    if len(tris) == 0:
        raise ValueError(f"{path}: no triangles")
    index = {int(t): k for k, t in enumerate(tags)}
    tri = np.vectorize(lambda t: index[int(t)], otypes=[np.int64])(tris)
    used = np.unique(tri)
    remap = -np.ones(len(tags), dtype=np.int64)
    remap[used] = np.arange(len(used))
    pts = xyz[used].copy()
    if bathymetry is not None:
        pts[:, 2] = bathymetry(pts[:, 0], pts[:, 1])
    return build_topology(pts, remap[tri])


def dump_fields(mesh: Mesh, prim, path: str) -> None:
    """w, hu, hv of every cell, one line each, tab-separated (h = w - b with
    b the centroid bathymetry)."""
    prim = np.asarray(prim, dtype=np.float64).reshape(mesh.num_cells, 3)
    h = prim[:, 0] - mesh.centroids()[:, 2]
    out = np.stack([prim[:, 0], h * prim[:, 1], h * prim[:, 2]], axis=1)
    with open(path, "w") as fh:
        for w, hu, hv in out:
            fh.write(f"{float(w)!r}\t{float(hu)!r}\t{float(hv)!r}\n")


def dump_domain(mesh: Mesh, geometry_path: str, topology_path: str) -> None:
    """Node x, y, z per line; then the number of edges, each edge's two nodes
    and two cells; the number of cells, each cell's nodes, edges and
    neighbours (walls are -1)."""
    with open(geometry_path, "w") as fh:
        for x, y, z in mesh.geometry:
            fh.write(f"{float(x)!r}\t{float(y)!r}\t{float(z)!r}\n")
    with open(topology_path, "w") as fh:
        fh.write(f"{mesh.num_edges}\n")
        for (a, b), (c, d) in zip(mesh.edge_nodes, mesh.edge_cells):
            fh.write(f"{a}\t{b}\t{c}\t{d}\n")
        fh.write(f"{mesh.num_cells}\n")
        for p, e, t in zip(mesh.cell_nodes, mesh.cell_edges, mesh.cell_neighbours):
            fh.write("\t".join(str(int(v)) for v in (*p, *e, *t)) + "\n")


def load_domain(geometry_path: str, topology_path: str) -> Mesh:
    """The inverse of dump_domain."""
    return load_reference_dump(geometry_path, topology_path)


def mesh_fingerprint(mesh: Mesh) -> str:
    """SHA-256 of the mesh's geometry and topology arrays (their bytes in the
    reference's layouts)."""
    h = hashlib.sha256()
    m = mesh.contiguous()
    for a in (m.geometry, m.edge_nodes, m.edge_cells, m.cell_nodes, m.cell_edges, m.cell_neighbours):
        h.update(np.asarray(a).tobytes())
    return h.hexdigest()


class State(NamedTuple):
    prim: np.ndarray   # (C, 3) primitive field
    time: float        # simulated time
    step: int          # steps taken
    cfl_ratio: float   # the CFL ratio the next step's dt comes from (nan: not recorded)


def save_state(path: str, mesh: Mesh, prim, t: float = 0.0, step: int = 0, cfl_ratio: float = float("nan")) -> None:
    """A checkpoint: the (C, 3) primitive field, the simulated time, the step
    count, the CFL ratio of the last flux pass and the mesh fingerprint
    (``.npz``; values stored bit for bit)."""
    prim = np.ascontiguousarray(prim, dtype=np.float64).reshape(mesh.num_cells, 3)
    with open(path, "wb") as fh:
        np.savez(fh, prim=prim, time=np.float64(t), step=np.int64(step), cfl_ratio=np.float64(cfl_ratio),
                 fingerprint=np.array(mesh_fingerprint(mesh)))


def load_state(path: str, mesh: Mesh = None) -> State:
    """The checkpoint's State; with ``mesh`` given, refuses a checkpoint
    written for another mesh."""
    with np.load(path) as z:
        if mesh is not None and str(z["fingerprint"]) != mesh_fingerprint(mesh):
            raise ValueError(f"{path}: checkpoint belongs to another mesh")
        return State(z["prim"].copy(), float(z["time"]), int(z["step"]), float(z["cfl_ratio"]))
