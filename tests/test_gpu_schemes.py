"""Time-scheme plugin: a caller's Shu-Osher table (swe_set_scheme) runs through
the same generic stage loop as the built-in schemes. Tables equal to Euler,
SSPRK2 and SSPRK3 reproduce them bit for bit; a four-stage SSPRK(4,2) matches
the CPU restatement bit for bit, in a batch too; its discrete adjoint matches
central finite differences."""
import ctypes

import numpy as np
import pytest

from oracle.oracle import JACOBI, Oracle
from swe_fvm_gb300 import Batch, Fluxes, Solvers, SpaceDisc, TimeDisc, Wavespeeds, _lib, scenarios
from swe_fvm_gb300.adjoint import Rollout
from swe_fvm_gb300.solver import ssprk_m2

pytestmark = pytest.mark.gpu

TABLES = {
    0: ([1.0], [0.0], [1.0]),
    1: ([1.0, 0.5], [0.0, 0.5], [1.0, 0.5]),
    2: ([1.0, 0.75, 1.0 / 3.0], [0.0, 0.25, 2.0 / 3.0], [1.0, 0.25, 2.0 / 3.0]),
}


@pytest.mark.parametrize("scheme", [0, 1, 2])
def test_builtin_tables_reproduce_the_builtin_schemes(gpu, scheme):
    m, prim = scenarios.random_front_case(24, 1)
    a = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, cfl=0.3)
    b = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, cfl=0.3)
    b.set_scheme(*TABLES[scheme])
    ta = a.run_cfl(scheme, 15)
    tb = b.run_cfl(Solvers.CUSTOM, 15)
    assert np.array_equal(a.GetVolField(), b.GetVolField())
    assert ta == tb


def test_four_stage_ssp_scheme_matches_the_oracle(gpu):
    m, prim = scenarios.random_front_case(24, 2)
    table = ssprk_m2(4)
    o = Oracle(m, prim, flux="HLLC", wavespeed="Einfeldt", order=JACOBI)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    sd.set_scheme(*table)
    td = TimeDisc(sd)
    o.compute_interface_values()
    o.compute_fluxes()
    for _ in range(8):
        dt = 0.15 * o.min_len_to_wavespeed()
        assert dt == td.CFLdt()
        o.step_table(*table, 3.0 * dt)  # SSP coefficient 3
        Solvers.Custom(td, 3.0 * dt)
        assert np.array_equal(sd.GetVolField(), o.prim())


def test_batch_custom_scheme_equals_single(gpu):
    cases = [scenarios.random_front_case(16, 3), scenarios.random_front_case(20, 4)]
    table = ssprk_m2(3)
    b = Batch([c[0] for c in cases], [c[1] for c in cases], Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.6)
    b.set_scheme(*table)
    b.run_cfl(Solvers.CUSTOM, 10)
    for q, (m, p) in enumerate(cases):
        sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p, cfl=0.6)
        sd.set_scheme(*table)
        t = sd.run_cfl(Solvers.CUSTOM, 10)
        assert np.array_equal(b.prim(q), sd.GetVolField()), q
        assert b.time(q) == t


def test_bad_tables_and_undefined_custom_scheme_are_rejected(gpu):
    m, prim = scenarios.lake_at_rest(6)
    sd = SpaceDisc(Fluxes.HLLC(), m, prim)
    L = _lib.load()
    assert L.swe_step(sd.ctx, 3, 1e-3) == 1  # not defined yet
    for a, b, c in (([0.5], [0.4], [1.0]), ([1.0], [0.0], [0.0]), ([1.0], [0.0], [float("nan")]),
                    ([1.0] * 5, [0.0] * 5, [1.0] * 5), ([], [], [])):
        a, b, c = (np.array(x, dtype=np.float64) for x in (a, b, c))
        st = L.swe_set_scheme(sd.ctx, a.size, a.ctypes.data, b.ctypes.data, c.ctypes.data)
        assert st == 1, (a, b, c)
    sd.set_scheme(*ssprk_m2(2))
    assert L.swe_step(sd.ctx, 3, 1e-3) == 0


def test_custom_scheme_adjoint_matches_central_differences(gpu):
    m, prim = scenarios.sloped_bump_case(25, 9)
    m = m.contiguous()
    gauges = np.random.default_rng(5).choice(m.num_cells, 12, replace=False)
    table = ssprk_m2(3)
    n_steps, obs, ckpt = 16, 4, 6
    ro = Rollout(m, prim, cfl=0.3)
    ro.sd.set_scheme(*table)
    traces = ro.forward(Solvers.CUSTOM, n_steps, ckpt, gauges, obs)
    dts = ro.dts(n_steps)
    target = traces * 0.97 + 0.002
    gp, gz = ro.backward(2.0 * (traces - target))

    def loss(p):
        sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p, cfl=0.3)
        sd.set_scheme(*table)
        td = TimeDisc(sd)
        out = []
        for n, dt in enumerate(dts):
            Solvers.Custom(td, dt)
            if (n + 1) % obs == 0:
                out.append(sd.GetVolField()[gauges, 0])
        return float(np.sum((np.array(out) - target) ** 2))

    assert loss(prim) == float(np.sum((traces - target) ** 2))
    bc = m.centroids()[:, 2]
    wet = np.where(prim[:, 0] - bc > 0.02)[0]
    cand = wet[np.argsort(-np.abs(gp[wet, 0]))[:5]]
    eps = 1e-7
    errs = []
    for c in cand:
        p1 = prim.copy(); p1[c, 0] += eps
        p2 = prim.copy(); p2[c, 0] -= eps
        fd = (loss(p1) - loss(p2)) / (2 * eps)
        errs.append(abs(gp[c, 0] - fd) / max(abs(fd), 1e-30))
    # central differences at eps = 1e-7 of a bit-deterministic forward: 1e-6
    # relative away from limiter, wet/dry and HLLC branch switches
    assert max(errs) < 1e-6, errs
