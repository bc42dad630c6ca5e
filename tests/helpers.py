"""Shared comparison helpers for the parity tests."""
import numpy as np


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def max_abs(a, b) -> float:
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b)))) if np.size(a) else 0.0


def cons(prim, bc):
    h = prim[:, 0] - bc
    return np.stack([h, h * prim[:, 1], h * prim[:, 2]], axis=1)



def shuffle_mesh(m, seed):
    """The same mesh with its cells, edges and nodes renumbered at random
    (each cell's and edge's own row order kept).  Returns (mesh, pc, pe, pn),
    p*[new] = old index."""
    from swe_fvm_gb300.mesh import shuffled

    return shuffled(m, seed)


GOLDEN = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)), "golden")


def read_bowl_mesh():
    """The reference's own examples/bowl.msh (kept gzipped in tests/golden),
    read by the library's Gmsh reader."""
    import gzip
    import os
    import tempfile

    from swe_fvm_gb300 import fileio

    with gzip.open(os.path.join(GOLDEN, "bowl.msh.gz"), "rb") as fh, tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "bowl.msh")
        with open(path, "wb") as out:
            out.write(fh.read())
        return fileio.read_gmsh(path)


def load_reference_vectors(name):
    """(mesh, prim0, data) of tests/golden/ref_<name>.npz, the golden vectors
    written by the reference's own solver (tests/golden/make_ref_fixtures.py)."""
    import os

    from swe_fvm_gb300.mesh import Mesh

    d = dict(np.load(os.path.join(GOLDEN, f"ref_{name}.npz")))
    if "geometry" in d:
        m = Mesh(d["geometry"], *(d[k].astype(np.int64) for k in ("edge_nodes", "edge_cells", "cell_nodes",
                                                                    "cell_edges", "cell_neighbours")))
        prim0 = d["prim0"]
    else:  # bowl: the mesh is read again from the reference's .msh file, flat bed
        m = read_bowl_mesh()
        m.geometry[:, 2] = 0.0
        prim0 = np.zeros((m.num_cells, 3))
        prim0[:, 0] = d["w0"]
    return m, prim0, d
