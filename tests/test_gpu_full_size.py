"""The benchmark configurations at their full sizes: the 1M-triangle dam break
against the CPU restatement bit for bit (two SSPRK2 steps, the restatement on
every host thread), then size-independent properties over a longer run
(positivity, volume conservation to round-off, determinism); lake at rest on a
524k-cell mesh; and members of the 256-instance ensemble batched equal to
their single contexts."""
import os

import numpy as np
import pytest

from oracle.oracle import JACOBI, Oracle
from swe_fvm_gb300 import Batch, Fluxes, Solvers, SpaceDisc, TimeDisc, Wavespeeds, scenarios

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dam():
    return scenarios.dam_break(708)


def _threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def test_dam_break_1m_equals_the_restatement(gpu, dam):
    m, prim = dam
    assert m.num_cells > 990_000
    o = Oracle(m, prim, flux="HLLC", wavespeed="Einfeldt", order=JACOBI)
    o.set_threads(_threads())
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    td = TimeDisc(sd)
    o.compute_interface_values()
    o.compute_fluxes()
    for _ in range(2):
        dt = 0.15 * o.min_len_to_wavespeed()
        assert dt == td.CFLdt()
        o.step("SSPRK2", dt)
        Solvers.SSPRK2(td, dt)
        assert np.array_equal(sd.GetVolField(), o.prim())


def test_dam_break_1m_properties(gpu, dam):
    """300 CFL steps: depth never negative (exact comparisons with the cell
    bathymetry), volume conserved to round-off (closed walls), and a second
    context reproduces the run bit for bit."""
    m, prim = dam
    bc = m.centroids()[:, 2]
    a = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    v0 = a.integrals()[0]
    for _ in range(3):
        a.run_cfl(1, 100)
        p = a.GetVolField()
        assert np.all(p[:, 0] - bc >= 0.0)
        assert np.all(np.isfinite(p))
    a.synchronize()
    v1 = a.integrals()[0]
    assert abs(v1 - v0) <= 1e-10 * v0, (v0, v1)
    b = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    b.run_cfl(1, 300)
    assert np.array_equal(a.GetVolField(), b.GetVolField())
    assert a.time() == b.time() > 0.0


def test_lake_at_rest_524k(gpu):
    m, prim = scenarios.lake_at_rest(512)
    assert m.num_cells == 2 * 512 * 512
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    sd.run_cfl(1, 100)
    p = sd.GetVolField()
    assert np.max(np.abs(p[:, 0] - prim[:, 0])) < 1e-12
    assert np.max(np.abs(p[:, 1:])) < 1e-12


def test_ensemble_256_members_equal_single_contexts(gpu):
    """The full ensemble (256 instances, 2k-200k cells, 11M cells) in one
    batch; the smallest, the largest and two others equal their single runs."""
    ens = scenarios.ensemble(256)
    fl = Fluxes.HLLC(Wavespeeds.Einfeldt)
    b = Batch([e[0] for e in ens], [e[1] for e in ens], fl, cfl=0.4)
    b.run_cfl(1, 6)
    b.synchronize()
    sizes = np.array([e[0].num_cells for e in ens])
    for q in sorted({int(np.argmin(sizes)), int(np.argmax(sizes)), 17, 200}):
        m, p = ens[q]
        sd = SpaceDisc(fl, m, p, cfl=0.4)
        t = sd.run_cfl(1, 6)
        assert np.array_equal(b.prim(q), sd.GetVolField()), q
        assert b.time(q) == t, q
