"""The GPU step against golden vectors written by the reference's own solver.

tests/golden/ref_*.npz hold states reached by the reference's src/*.cpp
(NikitaMatckevich/SWE_FVM, compiled by oracle/ref/build_ref.py with the Q1 and
Q20 edits) in jacobi loop order, written by tests/golden/make_ref_fixtures.py.
Each case is replayed here through the library's public API (SpaceDisc /
TimeDisc / Solvers, run_cfl) on cuda:0.

Tolerance: the target bounds, per-step relative L2 <= 1e-12 and final-time
relative L2 <= 1e-10, are asserted, and so is exact equality (the device path
computes in the reference's operation order, so every coefficient matches).
"""
import numpy as np
import pytest

from swe_fvm_gb300 import Fluxes, Solvers, SpaceDisc, TimeDisc, Wavespeeds
from tests.helpers import load_reference_vectors, rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-12
FINAL_TOL = 1e-10
WS = {"Rusanov": Wavespeeds.Rusanov, "Davis": Wavespeeds.Davis, "Einfeldt": Wavespeeds.Einfeldt}


def fluxer(flux, ws):
    return (Fluxes.HLLC if flux == "HLLC" else Fluxes.HLL)(WS[ws])


def assert_equal(a, b, tol, what):
    err = rel_l2(a, b)
    assert err <= tol, f"{what}: relative L2 {err:.3e}"
    n = int(np.count_nonzero(np.asarray(a) != np.asarray(b)))
    assert n == 0, f"{what}: {n} coefficients differ (relative L2 {err:.3e})"


def cfl_replay(m, prim0, d, flux, prefix=""):
    """run_cfl from a fresh context, checked at every stored step."""
    sd = SpaceDisc(fluxer(flux, "Einfeldt"), m, prim0, cfl=float(d["cfl"]))
    sd.ComputeInterfaceValues()
    sd.ComputeFluxes()
    done = 0
    for s in (int(x) for x in d["snaps"]):
        t = sd.run_cfl(Solvers.SSPRK2_ID, s - done)
        done = s
        tol = STEP_TOL if s == 1 else FINAL_TOL
        assert_equal(sd.GetVolField(), d[f"{prefix}prim_{s}"], tol, f"step {s}")
        assert t == pytest.approx(float(d[f"{prefix}t_{s}"]), rel=1e-14)


def test_thacker_8192_cells_1000_steps_equal_reference(gpu):
    """Workload: Thacker bowl 64 x 64 x 2, HLLC + Einfeldt, SSPRK2, CFL 0.4,
    1000 steps (graph-replayed, dt from the device CFL reduction)."""
    m, prim0, d = load_reference_vectors("thacker64")
    cfl_replay(m, prim0, d, "HLLC")


@pytest.mark.parametrize("flux", ["HLLC", "HLL"])
def test_dam_break_fronts_100_steps_equal_reference(gpu, flux):
    m, prim0, d = load_reference_vectors("dam_front")
    cfl_replay(m, prim0, d, flux, f"{flux}_")


def test_reference_driver_case_on_bowl_mesh(gpu):
    """examples/Main.cpp:172-195 on examples/bowl.msh: HLL + Einfeldt, Euler,
    dt = 1e-3, read through the library's Gmsh reader."""
    m, prim0, d = load_reference_vectors("bowl_gauss")
    sd = SpaceDisc(fluxer("HLL", "Einfeldt"), m, prim0)
    td = TimeDisc(sd)
    for _ in range(int(d["steps"])):
        Solvers.Euler(td, float(d["dt"]))
    assert_equal(sd.GetVolField(), d[f"prim_{int(d['steps'])}"], FINAL_TOL, "final state")


@pytest.mark.parametrize("scheme", ["Euler", "SSPRK2", "SSPRK3"])
@pytest.mark.parametrize("flux,ws", [(f, w) for f in ("HLL", "HLLC") for w in ("Rusanov", "Davis", "Einfeldt")])
def test_flux_plugins_and_schemes_equal_reference(gpu, flux, ws, scheme):
    m, prim0, d = load_reference_vectors("front_plugins")
    sd = SpaceDisc(fluxer(flux, ws), m, prim0)
    td = TimeDisc(sd)
    step = getattr(Solvers, scheme)
    for _ in range(int(d["steps"])):
        step(td, float(d["dt"]))
    assert_equal(sd.GetVolField(), d[f"{flux}_{ws}_{scheme}"], STEP_TOL, f"{flux}+{ws} {scheme}")


def test_interface_values_equal_reference(gpu):
    """ComputeInterfaceValues + ComputeFluxes of the initial state: edge values,
    source slots, node maxima, fluxes and the CFL ratio, in the reference's
    slot layout (2e + (from < to))."""
    m, prim0, d = load_reference_vectors("front_plugins")
    sd = SpaceDisc(fluxer("HLLC", "Einfeldt"), m, prim0)
    sd.ComputeInterfaceValues()
    sd.ComputeFluxes()
    assert_equal(sd.GetEdgField(), d["edg"], STEP_TOL, "edge values")
    assert_equal(sd.GetSrcField()[:, 1:], d["src"], STEP_TOL, "source slots")
    assert_equal(sd.GetNodeMax(), d["max_wp"], STEP_TOL, "node maxima")
    assert_equal(sd.GetFluxes(), d["fluxes"], STEP_TOL, "fluxes")
    assert sd.GetMinLenToWavespeed() == float(d["ratio"])


def test_coriolis_equal_reference(gpu):
    m, prim0, d = load_reference_vectors("front_plugins")
    sd = SpaceDisc(fluxer("HLLC", "Einfeldt"), m, prim0, cor=0.7)
    td = TimeDisc(sd)
    for _ in range(5):
        Solvers.SSPRK3(td, float(d["dt"]))
    assert_equal(sd.GetVolField(), d["coriolis_SSPRK3"], STEP_TOL, "Coriolis")
