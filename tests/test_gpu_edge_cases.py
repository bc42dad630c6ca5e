"""Edge cases of the step against the CPU restatement, bit for bit: a single
triangle (three walls), two cells, a domain that is dry everywhere, films at
the wet-depth thresholds, and a batch mixing one-cell and larger instances."""
import numpy as np
import pytest

from oracle.oracle import JACOBI, Oracle
from swe_fvm_gb300 import Batch, Fluxes, Solvers, SpaceDisc, TimeDisc, Wavespeeds, scenarios
from swe_fvm_gb300.mesh import build_topology

pytestmark = pytest.mark.gpu


def one_triangle():
    pts = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.1], [0.0, 1.0, 0.3]])
    m = build_topology(pts, np.array([[0, 1, 2]]))
    prim = np.array([[0.5, 0.2, -0.1]])
    return m, prim


def two_cells():
    pts = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.05], [1.0, 1.0, 0.2], [0.0, 1.0, 0.1]])
    m = build_topology(pts, np.array([[0, 1, 2], [0, 2, 3]]))
    prim = np.array([[0.4, 0.1, 0.0], [0.15, -0.2, 0.3]])
    return m, prim


def dry_everywhere():
    m, prim = scenarios.random_front_case(16, 4)
    prim = prim.copy()
    prim[:, 0] = m.centroids()[:, 2]
    prim[:, 1:] = 0.0
    return m, prim


def thin_films():
    """Depths around the 1e-12 wet threshold and the 1e-10 flux capture."""
    m, prim = scenarios.random_front_case(16, 6)
    prim = prim.copy()
    rng = np.random.default_rng(8)
    h = 10.0 ** rng.uniform(-13, -9, m.num_cells)
    prim[:, 0] = m.centroids()[:, 2] + h
    prim[:, 1:] = rng.normal(0, 0.01, (m.num_cells, 2))
    return m, prim


CASES = {"one_triangle": one_triangle, "two_cells": two_cells, "dry_everywhere": dry_everywhere,
         "thin_films": thin_films}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("scheme", ["Euler", "SSPRK2"])
def test_edge_case_steps_bit_exact(gpu, name, scheme):
    m, prim = CASES[name]()
    o = Oracle(m, prim, flux="HLLC", wavespeed="Einfeldt", order=JACOBI)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    td = TimeDisc(sd)
    o.compute_interface_values()
    o.compute_fluxes()
    for _ in range(6):
        dt = 0.15 * o.min_len_to_wavespeed()
        assert dt == td.CFLdt()
        o.step(scheme, dt)
        getattr(Solvers, scheme)(td, dt)
        assert np.array_equal(sd.GetVolField(), o.prim())
    if name == "dry_everywhere":
        # nothing moves; the CFL ratio keeps its reset value 1
        assert np.array_equal(sd.GetVolField(), prim)
        assert td.CFLdt() == 0.15


def test_batch_with_one_cell_instances_equals_single(gpu):
    cases = [one_triangle(), scenarios.random_front_case(12, 2), two_cells(), one_triangle()]
    b = Batch([c[0] for c in cases], [c[1] for c in cases], Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.3)
    b.run_cfl(1, 8)
    for q, (m, p) in enumerate(cases):
        sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p, cfl=0.3)
        t = sd.run_cfl(1, 8)
        assert np.array_equal(b.prim(q), sd.GetVolField()), q
        assert b.time(q) == t
