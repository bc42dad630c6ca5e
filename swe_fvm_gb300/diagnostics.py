"""Accuracy and conservation monitoring.

- ``SpaceDisc.integrals()`` / ``Batch.integrals(q)``: volume and energies
  summed on the device (swe_integrals).
- ``l2_errors``: the L2 norm over the domain of the error in (h, hu, hv)
  against a closed-form solution, sqrt(sum_i A_i e_i^2) (the reference's
  Compare + OutputL2Errors, src/SpaceDisc.cpp:106-139 and
  examples/Main.cpp:47-61, both commented out there).  The reference takes e_i
  as the cell average of |exact - reconstruction|; here e_i is
  |TriangAverage(exact) - cell average|, so the norm measures the cell
  averages the solver evolves.
"""
from __future__ import annotations

import numpy as np

from .analytic import Solution, cell_averages
from .mesh import Mesh

__all__ = ["l2_errors", "conserved"]


def conserved(mesh: Mesh, prim) -> np.ndarray:
    """(h, hu, hv) per cell from the primitive state (w, u, v)."""
    prim = np.asarray(prim, dtype=np.float64).reshape(mesh.num_cells, 3)
    h = np.maximum(prim[:, 0] - mesh.centroids()[:, 2], 0.0)
    return np.stack([h, h * prim[:, 1], h * prim[:, 2]], axis=1)


def l2_errors(mesh: Mesh, prim, sol: Solution, t: float, n: int = 10) -> np.ndarray:
    """(3,) L2 errors of (h, hu, hv) at time t, quadrature TriangAverage<3, n>."""
    exact = cell_averages(mesh, sol, t, n)
    err = np.abs(exact - conserved(mesh, prim))
    return np.sqrt(mesh.areas() @ (err * err))
