"""Mesh ingestion and the reference's text outputs.

- ``read_gmsh`` / ``write_gmsh``: Gmsh meshes (format 2.2 or 4.1, ASCII or
  binary) to and from the reference's topology (notebooks/mesher.py:3-69 reads
  them through the gmsh API; gmsh is not needed here).  Triangles (element
  type 2) become cells; node z is the bathymetry; every edge with one cell is
  a solid wall.
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
import re
import struct
from typing import NamedTuple

import numpy as np

from .mesh import Mesh, build_topology, load_reference_dump

__all__ = ["read_gmsh", "write_gmsh", "dump_fields", "dump_domain", "load_domain", "save_state", "load_state",
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


# nodes per element of the Gmsh element types a 2-D or 3-D mesh file may carry
_NODES_PER_TYPE = {1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 6: 6, 7: 5, 8: 3, 9: 6, 10: 9, 11: 10, 12: 27, 13: 18, 14: 14,
                   15: 1, 16: 8, 17: 20, 18: 15, 19: 13, 20: 9, 21: 10, 22: 12, 23: 15, 24: 15, 25: 21, 26: 4,
                   27: 5, 28: 6, 29: 20, 30: 35, 31: 56, 92: 64, 93: 125}


def _binary_body(data: bytes, name: str, path: str, start: int = 0) -> int:
    """Offset of the first byte after the '$name' line, searched from `start`
    (the end of the section read before it, so that binary payloads already
    walked over cannot match) at the start of a line, LF or CRLF."""
    m = re.compile(rb"(?:\A|(?<=\n))\$" + re.escape(name.encode()) + rb"\r?\n").search(data, start)
    if m is None:
        raise ValueError(f"{path}: no ${name} section")
    return m.end()


def _nodes_start(data: bytes, path: str) -> int:
    """Where to look for $Nodes: after $EndMeshFormat, and after the binary
    $Entities / $PartitionedEntities sections when present."""
    pos = _binary_body(data, "EndMeshFormat", path)
    for sec in ("EndEntities", "EndPartitionedEntities"):
        m = re.compile(rb"(?:\A|(?<=\n))\$" + sec.encode() + rb"\r?\n").search(data, pos)
        if m is not None:
            pos = m.end()
    return pos


def _gmsh_binary(data: bytes, version: str, dsize: int, path: str):
    """Binary Gmsh 2.2 / 4.1: nodes (tags, xyz) and the triangles' node tags."""
    pos = _binary_body(data, "MeshFormat", path)
    pos = data.index(b"\n", pos) + 1  # the "version 1 size" line
    if struct.unpack_from("<i", data, pos)[0] == 1:
        e = "<"
    elif struct.unpack_from(">i", data, pos)[0] == 1:
        e = ">"
    else:
        raise ValueError(f"{path}: unreadable binary header")
    st = {4: "i4", 8: "i8"}.get(dsize)
    if st is None:
        raise ValueError(f"{path}: data size {dsize} is not supported")
    st, i4, f8 = np.dtype(e + st), np.dtype(e + "i4"), np.dtype(e + "f8")
    if version.startswith("4"):
        pos = _binary_body(data, "Nodes", path, _nodes_start(data, path))
        n_blocks = int(np.frombuffer(data, st, 4, pos)[0])
        pos += 4 * dsize
        tags, coords = [], []
        for _ in range(n_blocks):
            dim, _tag, parametric = (int(v) for v in np.frombuffer(data, i4, 3, pos))
            count = int(np.frombuffer(data, st, 1, pos + 12)[0])
            pos += 12 + dsize
            tags.append(np.frombuffer(data, st, count, pos).astype(np.int64))
            pos += count * dsize
            width = 3 + (dim if parametric else 0)
            coords.append(np.frombuffer(data, f8, count * width, pos).reshape(count, width)[:, :3])
            pos += count * width * 8
        pos = _binary_body(data, "Elements", path, pos)
        n_blocks = int(np.frombuffer(data, st, 4, pos)[0])
        pos += 4 * dsize
        tris = []
        for _ in range(n_blocks):
            _dim, _tag, etype = (int(v) for v in np.frombuffer(data, i4, 3, pos))
            count = int(np.frombuffer(data, st, 1, pos + 12)[0])
            pos += 12 + dsize
            if etype not in _NODES_PER_TYPE:
                raise ValueError(f"{path}: element type {etype} is not supported")
            width = 1 + _NODES_PER_TYPE[etype]
            rows = np.frombuffer(data, st, count * width, pos).reshape(count, width)
            if etype == 2:
                tris.append(rows[:, 1:4].astype(np.int64))
            pos += count * width * dsize
        xyz = np.concatenate(coords) if coords else np.zeros((0, 3))
        tags = np.concatenate(tags) if tags else np.zeros(0, np.int64)
        tris = np.concatenate(tris) if tris else np.zeros((0, 3), np.int64)
        return tags, xyz, tris
    # 2.2: the counts are text lines, the records binary
    pos = _binary_body(data, "Nodes", path, _nodes_start(data, path))
    end = data.index(b"\n", pos)
    n = int(data[pos:end])
    rec = np.dtype([("tag", i4), ("xyz", f8, (3,))])
    nodes = np.frombuffer(data, rec, n, end + 1)
    pos = _binary_body(data, "Elements", path, end + 1 + n * rec.itemsize)
    end = data.index(b"\n", pos)
    remaining = int(data[pos:end])
    pos = end + 1
    tris = []
    while remaining > 0:
        etype, count, ntags = (int(v) for v in np.frombuffer(data, i4, 3, pos))
        pos += 12
        if etype not in _NODES_PER_TYPE or count <= 0:
            raise ValueError(f"{path}: bad element block (type {etype}, {count} elements)")
        width = 1 + ntags + _NODES_PER_TYPE[etype]
        rows = np.frombuffer(data, i4, count * width, pos).reshape(count, width)
        if etype == 2:
            tris.append(rows[:, 1 + ntags:4 + ntags].astype(np.int64))
        pos += count * width * 4
        remaining -= count
    tris = np.concatenate(tris) if tris else np.zeros((0, 3), np.int64)
    return nodes["tag"].astype(np.int64), np.array(nodes["xyz"], dtype=np.float64), tris


def read_gmsh(path: str, bathymetry=None) -> Mesh:
    """Gmsh mesh (format 2.2 or 4.1, ASCII or binary) -> Mesh.  bathymetry(x,
    y), if given, replaces the node z.  Nodes not used by any triangle are
    dropped; the rest keep the file's order."""
    with open(path, "rb") as fh:
        data = fh.read()
    head = data[:256].decode("latin-1")
    if "$MeshFormat" not in head:
        raise ValueError(f"{path}: no $MeshFormat section")
    fmt = head.split("$MeshFormat", 1)[1].split()
    if len(fmt) < 3:
        raise ValueError(f"{path}: malformed $MeshFormat")
    version, binary, dsize = fmt[0], fmt[1], int(fmt[2])
    if not (version.startswith("2") or version.startswith("4")):
        raise ValueError(f"{path}: Gmsh format {version} is not supported (2.2 or 4.1)")
    if binary != "0":
        try:
            tags, xyz, tris = _gmsh_binary(data, version, dsize, path)
        except (IndexError, ValueError, struct.error) as ex:
            raise ValueError(f"{path}: {ex}") from None
    else:
        sec = _sections(data.decode("latin-1"))
        tags, xyz, tris = (_gmsh2 if version.startswith("2") else _gmsh4)(sec)
    if len(tris) == 0:
        raise ValueError(f"{path}: no triangles")
    # node tag -> position in the file, vectorised
    tags = np.asarray(tags, dtype=np.int64)
    if len(tags) == 0:
        raise ValueError(f"{path}: no nodes")
    order = np.argsort(tags, kind="stable")
    at = np.searchsorted(tags[order], tris)
    at = np.minimum(at, len(tags) - 1)
    tri = order[at]
    if not np.array_equal(tags[tri], tris):
        raise ValueError(f"{path}: a triangle names a node tag the file does not define")
    used = np.unique(tri)
    remap = -np.ones(len(tags), dtype=np.int64)
    remap[used] = np.arange(len(used))
    pts = xyz[used].copy()
    if bathymetry is not None:
        pts[:, 2] = bathymetry(pts[:, 0], pts[:, 1])
    return build_topology(pts, remap[tri])


def write_gmsh(path: str, mesh: Mesh, version: str = "4.1", binary: bool = False) -> None:
    """The mesh as a Gmsh file (format 2.2 or 4.1, ASCII or binary): its nodes
    (x, y, z with z the bathymetry, tags 1..N) and its triangles (tags 1..C),
    one block each, little-endian 8-byte sizes when binary."""
    xyz = np.ascontiguousarray(mesh.geometry, dtype="<f8")
    tri = np.ascontiguousarray(mesh.cell_nodes, dtype=np.int64) + 1
    N, C = len(xyz), len(tri)
    v4 = version.startswith("4")
    with open(path, "wb") as fh:
        fh.write(f"$MeshFormat\n{'4.1' if v4 else '2.2'} {1 if binary else 0} 8\n".encode())
        if binary:
            fh.write(np.array([1], "<i4").tobytes() + b"\n")
        fh.write(b"$EndMeshFormat\n$Nodes\n")
        if v4 and binary:
            fh.write(np.array([1, N, 1, N], "<u8").tobytes() + np.array([2, 1, 0], "<i4").tobytes()
                     + np.array([N], "<u8").tobytes() + np.arange(1, N + 1, dtype="<u8").tobytes() + xyz.tobytes())
        elif v4:
            fh.write(f"1 {N} 1 {N}\n2 1 0 {N}\n".encode())
            fh.write("".join(f"{k}\n" for k in range(1, N + 1)).encode())
            fh.write("".join(f"{float(x)!r} {float(y)!r} {float(z)!r}\n" for x, y, z in xyz).encode())
        elif binary:
            rec = np.zeros(N, np.dtype([("tag", "<i4"), ("xyz", "<f8", (3,))]))
            rec["tag"], rec["xyz"] = np.arange(1, N + 1), xyz
            fh.write(f"{N}\n".encode() + rec.tobytes())
        else:
            fh.write(f"{N}\n".encode())
            fh.write("".join(f"{k + 1} {float(x)!r} {float(y)!r} {float(z)!r}\n"
                             for k, (x, y, z) in enumerate(xyz)).encode())
        fh.write(b"\n$EndNodes\n$Elements\n" if binary else b"$EndNodes\n$Elements\n")
        ids = np.arange(1, C + 1, dtype=np.int64)
        if v4 and binary:
            fh.write(np.array([1, C, 1, C], "<u8").tobytes() + np.array([2, 1, 2], "<i4").tobytes()
                     + np.array([C], "<u8").tobytes() + np.column_stack([ids, tri]).astype("<u8").tobytes())
        elif v4:
            fh.write(f"1 {C} 1 {C}\n2 1 2 {C}\n".encode())
            fh.write("".join(f"{i} {a} {b} {c}\n" for i, (a, b, c) in zip(ids, tri)).encode())
        elif binary:
            body = np.column_stack([ids, np.ones(C, np.int64), tri]).astype("<i4")  # id, physical tag, nodes
            fh.write(f"{C}\n".encode() + np.array([2, C, 1], "<i4").tobytes() + body.tobytes())
        else:
            fh.write(f"{C}\n".encode())
            fh.write("".join(f"{i} 2 1 1 {a} {b} {c}\n" for i, (a, b, c) in zip(ids, tri)).encode())
        fh.write(b"\n$EndElements\n" if binary else b"$EndElements\n")


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
