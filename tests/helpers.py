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
