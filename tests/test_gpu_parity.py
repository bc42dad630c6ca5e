"""Parity of the sm_103a step with the CPU restatement (jacobi order).

Tolerances (FP64): per-step relative L2 of the primitive field <= 1e-12 and
final-time relative L2 <= 1e-10.  With the default build (no FMA fusion on the
device, the reference's operation order, correctly rounded division, square
and cube roots on both sides) the two agree bit for bit.
"""
import numpy as np
import pytest

from oracle.oracle import JACOBI, Oracle
from swe_fvm_gb300 import Batch, Fluxes, Solvers, SpaceDisc, TimeDisc, Wavespeeds, scenarios
from swe_fvm_gb300.solver import SweError
from tests.helpers import max_abs, rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-12
FINAL_TOL = 1e-10

FLUXES = {
    "HLLC-Einfeldt": ("HLLC", "Einfeldt", Fluxes.HLLC(Wavespeeds.Einfeldt)),
    "HLL-Einfeldt": ("HLL", "Einfeldt", Fluxes.HLL(Wavespeeds.Einfeldt)),
    "HLLC-Rusanov": ("HLLC", "Rusanov", Fluxes.HLLC(Wavespeeds.Rusanov)),
    "HLL-Davis": ("HLL", "Davis", Fluxes.HLL(Wavespeeds.Davis)),
    "HLLC-Davis": ("HLLC", "Davis", Fluxes.HLLC(Wavespeeds.Davis)),
    "HLL-Rusanov": ("HLL", "Rusanov", Fluxes.HLL(Wavespeeds.Rusanov)),
}

_CACHE = {}


def case(name):
    if name not in _CACHE:
        if name == "thacker16":
            _CACHE[name] = scenarios.thacker(16, quad=10)
        elif name == "front":
            _CACHE[name] = scenarios.random_front_case(24, seed=0)
        elif name == "front5":
            _CACHE[name] = scenarios.random_front_case(32, seed=5)
        elif name == "lake":
            _CACHE[name] = scenarios.lake_at_rest(12)
        elif name == "dam":
            _CACHE[name] = scenarios.dam_break(lattice=48)
        elif name == "hump":
            _CACHE[name] = scenarios.hump_instance(1003, 3000)
        else:
            raise KeyError(name)
    return _CACHE[name]


CASES = ["thacker16", "front", "front5", "lake", "dam", "hump"]


def pair(name, fkey="HLLC-Einfeldt", cor=0.0):
    m, prim = case(name)
    fl, ws, fluxer = FLUXES[fkey]
    o = Oracle(m, prim, flux=fl, wavespeed=ws, cor=cor, order=JACOBI)
    sd = SpaceDisc(fluxer, m, prim, cor=cor)
    return m, prim, o, sd


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("fkey", ["HLLC-Einfeldt", "HLL-Einfeldt"])
def test_interface_values_and_fluxes(gpu, name, fkey):
    """SpaceDisc::ComputeInterfaceValues + ComputeFluxes on the initial state."""
    m, prim, o, sd = pair(name, fkey)
    o.compute_interface_values()
    sd.ComputeInterfaceValues()
    edg_o, src_o, _, mx_o = o.edge_fields()
    assert rel_l2(sd.GetEdgField(), edg_o) <= STEP_TOL
    assert rel_l2(sd.GetSrcField(), src_o) <= STEP_TOL
    assert rel_l2(sd.GetNodeMax(), mx_o) <= STEP_TOL
    o.compute_fluxes()
    sd.ComputeFluxes()
    _, _, f_o, _ = o.edge_fields()
    f_g = sd.GetFluxes()
    assert rel_l2(f_g, f_o) <= STEP_TOL or max_abs(f_g, f_o) < 1e-15
    assert sd.GetMinLenToWavespeed() == pytest.approx(o.min_len_to_wavespeed(), rel=1e-14)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("scheme", ["Euler", "SSPRK2", "SSPRK3"])
def test_step_parity(gpu, name, scheme):
    """Ten steps with dt = 0.4 x the CFL ratio of the previous flux pass."""
    m, prim, o, sd = pair(name)
    td = TimeDisc(sd)
    o.compute_interface_values()
    o.compute_fluxes()
    step = getattr(Solvers, scheme)
    for s in range(10):
        dt = 0.4 * o.min_len_to_wavespeed()
        assert dt == pytest.approx(0.4 / 0.15 * td.CFLdt(), rel=1e-14)
        o.step(scheme, dt)
        step(td, dt)
        err = rel_l2(sd.GetVolField(), o.prim())
        assert err <= STEP_TOL, f"step {s}: relative L2 {err:.3e}"


@pytest.mark.parametrize("fkey", list(FLUXES))
def test_flux_plugins(gpu, fkey):
    """Every flux x wave-speed plugin on the wet/dry front case."""
    m, prim, o, sd = pair("front5", fkey)
    td = TimeDisc(sd)
    for s in range(6):
        o.step("SSPRK2", 2e-3)
        Solvers.SSPRK2(td, 2e-3)
        assert rel_l2(sd.GetVolField(), o.prim()) <= STEP_TOL


def test_coriolis(gpu):
    m, prim, o, sd = pair("front", cor=0.7)
    td = TimeDisc(sd)
    for s in range(5):
        o.step("SSPRK3", 2e-3)
        Solvers.SSPRK3(td, 2e-3)
        assert rel_l2(sd.GetVolField(), o.prim()) <= STEP_TOL


def test_thacker_8192_cells(gpu):
    """Workload: Thacker bowl, 64 x 64 x 2 cells, HLLC + Einfeldt, SSPRK2, CFL
    0.4, walls: per-step error for the first 10 steps, then 300 more steps
    through the graph-replayed CFL loop against the restatement's loop."""
    m, prim = scenarios.thacker(64, quad=20)
    o = Oracle(m, prim)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, cfl=0.4)
    td = TimeDisc(sd)
    o.compute_interface_values()
    o.compute_fluxes()
    t = 0.0
    for s in range(10):
        dt = 0.4 * o.min_len_to_wavespeed()
        o.step("SSPRK2", dt)
        Solvers.SSPRK2(td, dt)
        t += dt
        assert rel_l2(sd.GetVolField(), o.prim()) <= STEP_TOL
    for s in range(300):
        dt = 0.4 * o.min_len_to_wavespeed()
        o.step("SSPRK2", dt)
        t += dt
    tg = sd.run_cfl(1, 300)
    assert rel_l2(sd.GetVolField(), o.prim()) <= FINAL_TOL
    assert tg == pytest.approx(t, rel=1e-12)


def test_run_cfl_matches_restatement_loop(gpu):
    m, prim, o, sd = pair("dam")
    o.compute_interface_values()
    o.compute_fluxes()
    t = 0.0
    for s in range(25):
        dt = 0.15 * o.min_len_to_wavespeed()
        o.step("SSPRK2", dt)
        t += dt
    tg = sd.run_cfl(1, 25)
    assert rel_l2(sd.GetVolField(), o.prim()) <= FINAL_TOL
    assert tg == pytest.approx(t, rel=1e-13)


def test_fixed_dt_graph_run_equals_single_steps(gpu):
    m, prim = case("front")
    a = SpaceDisc(Fluxes.HLLC(), m, prim)
    b = SpaceDisc(Fluxes.HLLC(), m, prim)
    tda = TimeDisc(a)
    for _ in range(7):
        Solvers.SSPRK3(tda, 1e-3)
    b.run(2, 1e-3, 7)
    assert np.array_equal(a.GetVolField(), b.GetVolField())


def test_deterministic(gpu):
    m, prim = case("dam")
    outs = []
    for _ in range(2):
        sd = SpaceDisc(Fluxes.HLLC(), m, prim)
        sd.run_cfl(1, 20)
        outs.append(sd.GetVolField())
    assert np.array_equal(outs[0], outs[1])


def test_batch_equals_single_instances(gpu):
    """A batch of uneven instances gives, per instance, the same bits as the
    instance stepped alone, each with its own CFL time step."""
    cases = [case("front"), case("hump"), case("thacker16"), case("dam")]
    meshes = [c[0] for c in cases]
    prims = [c[1] for c in cases]
    b = Batch(meshes, prims, Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.3)
    b.run_cfl(1, 15)
    b.synchronize()
    for q, (m, p) in enumerate(cases):
        sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p, cfl=0.3)
        t = sd.run_cfl(1, 15)
        assert np.array_equal(b.prim(q), sd.GetVolField()), q
        assert b.time(q) == t


def test_positivity_and_lake_at_rest(gpu):
    m, prim = case("front5")
    bc = m.centroids()[:, 2]
    sd = SpaceDisc(Fluxes.HLLC(), m, prim)
    for _ in range(10):
        sd.run_cfl(1, 5)
        p = sd.GetVolField()
        assert np.all(p[:, 0] - bc >= 0.0)
    m, prim = case("lake")
    sd = SpaceDisc(Fluxes.HLLC(), m, prim)
    sd.run(1, 5e-3, 50)
    p = sd.GetVolField()
    assert np.max(np.abs(p[:, 0] - prim[:, 0])) < 1e-12
    assert np.max(np.abs(p[:, 1:])) < 1e-12


def test_errors_are_reported(gpu):
    m, prim = case("front")
    sd = SpaceDisc(Fluxes.HLLC(), m, prim)
    with pytest.raises(SweError) as ei:
        Solvers.SSPRK2(TimeDisc(sd), -1.0)
    assert ei.value.status == 1
    bad = prim.copy()
    bad[3, 0] = np.nan
    with pytest.raises(SweError) as ei:
        sd.SetVolField(bad)
    assert ei.value.status == 3
    with pytest.raises(SweError):
        SpaceDisc(Fluxes.HLLC(), m, bad)
