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


def test_adjoint_250k_linearity_and_tape(gpu):
    """The adjoint configuration's mesh (250k cells): the taped forward equals
    the plain steps bit for bit, and the backward pass is linear in the trace
    gradients (doubling is exact up to the order of the atomic node sums,
    superposition holds to round-off)."""
    from swe_fvm_gb300.adjoint import Rollout

    m, prim = scenarios.hump_instance(2024, 250_000)
    m = m.contiguous()
    gauges = np.random.default_rng(11).choice(m.num_cells, 64, replace=False)
    n, obs = 100, 10
    ro = Rollout(m, prim)
    tr = ro.forward(1, n, 50, gauges, obs)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    td = TimeDisc(sd)
    plain = []
    for k, dt in enumerate(ro.dts(n)):
        Solvers.SSPRK2(td, dt)
        if (k + 1) % obs == 0:
            plain.append(sd.GetVolField()[gauges, 0])
    assert np.array_equal(tr, np.array(plain))
    rng = np.random.default_rng(3)
    g1, g2 = rng.normal(size=tr.shape), rng.normal(size=tr.shape)
    p1, z1 = ro.backward(g1)
    p2, z2 = ro.backward(g2)
    p12, z12 = ro.backward(g1 + g2)
    pd, zd = ro.backward(2.0 * g1)
    for a, b in ((p1, pd), (z1, zd)):
        assert np.all(np.isfinite(a)) and np.max(np.abs(a)) > 0
        assert np.max(np.abs(2.0 * a - b)) <= 1e-13 * np.max(np.abs(b))
    for a, b, c in ((p1, p2, p12), (z1, z2, z12)):
        assert np.max(np.abs(a + b - c)) <= 1e-11 * np.max(np.abs(c))
