"""The C restatement pinned to the reference's own solver.

oracle/_ref/libswe_ref.so is the reference's src/*.cpp (NikitaMatckevich/
SWE_FVM) compiled here against the Eigen subset in oracle/eigen_subset, with
the two documented edits Q1 (src/Bathymetry.cpp:29-31, edge centre = midpoint)
and Q20 (src/MUSCLObject.cpp:68, vertex level minus that vertex's bathymetry),
built by oracle/ref/build_ref.py.  Its loop order is either the reference's
own (literal: Solvers::Euler/SSPRK2/SSPRK3 with in-place updates) or jacobi
(the same reference calls, every RHS of a stage evaluated before any write --
the order of the GPU path).

The restatement (oracle/swe_oracle.c) must equal it bit for bit in both
orders: interface values, source slots, node maxima, fluxes, CFL ratio and
the state after every step, for every flux plugin and time scheme, on meshes
with every reconstruction branch (tolerance written: exact equality; the
target bound, per-step relative L2 <= 1e-12, is implied).

The reference build needs the reference sources and is skipped where they are
absent; the golden vectors it wrote (tests/golden/ref_*.npz) are checked
against the restatement everywhere.
"""
import numpy as np
import pytest

from oracle import reference
from oracle.oracle import JACOBI, LITERAL, Oracle
from swe_fvm_gb300 import scenarios
from tests.helpers import load_reference_vectors, rel_l2

needs_ref = pytest.mark.skipif(not reference.available(), reason="the reference sources are not on this machine")

PLUGINS = [(f, w) for f in ("HLL", "HLLC") for w in ("Rusanov", "Davis", "Einfeldt")]
ORDERS = {"jacobi": JACOBI, "literal": LITERAL}

_CACHE = {}


def case(name):
    if name not in _CACHE:
        _CACHE[name] = {
            "front": lambda: scenarios.random_front_case(16, seed=2),
            "front5": lambda: scenarios.random_front_case(20, seed=5),
            "thacker16": lambda: scenarios.thacker(16, quad=10),
            "dam": lambda: scenarios.dam_break(lattice=16),
            "lake": lambda: scenarios.lake_at_rest(8),
            "sloped": lambda: scenarios.sloped_bump_case(12, 9),
            "hump": lambda: scenarios.hump_instance(1003, 800),
        }[name]()
    return _CACHE[name]


def both(name, flux="HLLC", ws="Einfeldt", order=JACOBI, cor=0.0):
    m, prim = case(name)
    r = reference.Reference(m, prim, flux, ws, cor=cor, order=order)
    o = Oracle(m, prim, flux=flux, wavespeed=ws, cor=cor, order=order)
    return m, prim, r, o


def assert_same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    n = int(np.count_nonzero(a != b))
    assert n == 0, f"{what}: {n} coefficients differ, relative L2 {rel_l2(a, b):.3e}"


@needs_ref
@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("name", ["front", "front5", "thacker16", "dam", "lake", "sloped", "hump"])
def test_interface_values_equal_reference(name, order):
    """SpaceDisc::ComputeInterfaceValues + ComputeFluxes of the initial state."""
    m, prim, r, o = both(name, order=ORDERS[order])
    r.interface()
    o.compute_interface_values()
    o.compute_fluxes()
    (er, sr, fr, mr), (eo, so, fo, mo) = r.edge_fields(), o.edge_fields()
    assert_same(er, eo, "edge values")
    assert_same(sr[:, 1:], so[:, 1:], "source slots")
    assert_same(fr, fo, "fluxes")
    assert_same(mr, mo, "node maxima")
    assert r.min_len_to_wavespeed() == o.min_len_to_wavespeed()
    assert_same(r.classify(), o.classify(), "cell classes")


@needs_ref
@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("scheme", ["Euler", "SSPRK2", "SSPRK3"])
@pytest.mark.parametrize("name", ["front", "thacker16", "dam", "sloped", "hump"])
def test_steps_equal_reference(name, scheme, order):
    """Eight steps, dt = 0.4 x the CFL ratio of the latest flux pass."""
    m, prim, r, o = both(name, order=ORDERS[order])
    r.interface()
    o.compute_interface_values()
    o.compute_fluxes()
    for s in range(8):
        assert r.min_len_to_wavespeed() == o.min_len_to_wavespeed(), s
        dt = 0.4 * o.min_len_to_wavespeed()
        r.step(scheme, dt)
        o.step(scheme, dt)
        assert_same(r.prim(), o.prim(), f"step {s}")


@needs_ref
@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("flux,ws", PLUGINS)
def test_flux_plugins_equal_reference(flux, ws, order):
    m, prim, r, o = both("front5", flux, ws, order=ORDERS[order])
    for s in range(5):
        r.step("SSPRK2", 2e-3)
        o.step("SSPRK2", 2e-3)
        assert_same(r.prim(), o.prim(), f"step {s}")
    assert r.min_len_to_wavespeed() == o.min_len_to_wavespeed()


@needs_ref
@pytest.mark.parametrize("order", ORDERS)
def test_coriolis_equal_reference(order):
    m, prim, r, o = both("front", cor=0.7, order=ORDERS[order])
    for s in range(5):
        r.step("SSPRK3", 2e-3)
        o.step("SSPRK3", 2e-3)
        assert_same(r.prim(), o.prim(), f"step {s}")


@needs_ref
@pytest.mark.parametrize("order", ORDERS)
def test_thacker_8192_cells_equal_reference(order):
    """Workload: Thacker bowl 64 x 64 x 2, HLLC + Einfeldt, SSPRK2, CFL 0.4."""
    m, prim = scenarios.thacker(64, quad=20)
    r = reference.Reference(m, prim, order=ORDERS[order])
    o = Oracle(m, prim, order=ORDERS[order])
    r.interface()
    o.compute_interface_values()
    o.compute_fluxes()
    for s in range(6):
        dt = 0.4 * o.min_len_to_wavespeed()
        r.step("SSPRK2", dt)
        o.step("SSPRK2", dt)
        assert_same(r.prim(), o.prim(), f"step {s}")


@needs_ref
def test_q20_edit_matters():
    """The positivity test as Eigen's release build reads src/MUSCLObject.cpp:68
    (node ip[0]'s x, y, z subtracted from the three vertex levels) changes the
    result on a mesh with fully wet cells next to emerging bumps; the
    restatement follows the edited reference, not that reading."""
    m, prim = case("front")
    lit = reference.Reference(m, prim, order=JACOBI, q20_literal=True)
    o = Oracle(m, prim, order=JACOBI)
    for s in range(5):
        lit.step("SSPRK2", 2e-3)
        o.step("SSPRK2", 2e-3)
    assert rel_l2(lit.prim(), o.prim()) > 1e-6


# ------------------------------------------------- golden vectors, anywhere
def test_restatement_reproduces_reference_vectors_front():
    m, prim0, d = load_reference_vectors("front_plugins")
    for f, w in PLUGINS:
        for s in ("Euler", "SSPRK2", "SSPRK3"):
            o = Oracle(m, prim0, flux=f, wavespeed=w)
            for _ in range(int(d["steps"])):
                o.step(s, float(d["dt"]))
            assert_same(o.prim(), d[f"{f}_{w}_{s}"], f"{f}+{w} {s}")
    o = Oracle(m, prim0)
    o.compute_interface_values()
    o.compute_fluxes()
    edg, src, f, mx = o.edge_fields()
    assert_same(edg, d["edg"], "edge values")
    assert_same(src[:, 1:], d["src"], "source slots")
    assert_same(f, d["fluxes"], "fluxes")
    assert_same(mx, d["max_wp"], "node maxima")
    assert o.min_len_to_wavespeed() == float(d["ratio"])
    assert_same(o.classify(), d["classes"], "cell classes")
    o = Oracle(m, prim0, cor=0.7)
    for _ in range(5):
        o.step("SSPRK3", float(d["dt"]))
    assert_same(o.prim(), d["coriolis_SSPRK3"], "Coriolis")


def _cfl_replay(m, prim0, d, flux, key_prefix=""):
    o = Oracle(m, prim0, flux=flux, wavespeed="Einfeldt")
    o.compute_interface_values()
    o.compute_fluxes()
    snaps = set(int(s) for s in d["snaps"])
    t = 0.0
    for s in range(1, int(d["steps"]) + 1):
        dt = float(d["cfl"]) * o.min_len_to_wavespeed()
        assert dt == d[f"{key_prefix}dts"][s - 1]
        o.step(str(d["scheme"]), dt)
        t += dt
        if s in snaps:
            assert_same(o.prim(), d[f"{key_prefix}prim_{s}"], f"step {s}")
            assert t == float(d[f"{key_prefix}t_{s}"])


def test_restatement_reproduces_reference_vectors_dam_front():
    m, prim0, d = load_reference_vectors("dam_front")
    for flux in ("HLLC", "HLL"):
        _cfl_replay(m, prim0, d, flux, f"{flux}_")


def test_restatement_reproduces_reference_vectors_bowl():
    """The reference's own driver case on its own mesh (examples/Main.cpp:172-195)."""
    m, prim0, d = load_reference_vectors("bowl_gauss")
    o = Oracle(m, prim0, flux="HLL", wavespeed="Einfeldt")
    for s in range(1, int(d["steps"]) + 1):
        o.step("Euler", float(d["dt"]))
    assert_same(o.prim(), d[f"prim_{int(d['steps'])}"], "final state")


def test_restatement_reproduces_reference_vectors_thacker_1000_steps():
    """Workload: Thacker 8192 cells, 1000 CFL-0.4 steps of the reference."""
    m, prim0, d = load_reference_vectors("thacker64")
    _cfl_replay(m, prim0, d, "HLLC")
