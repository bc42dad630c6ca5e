"""The C ABI library without a GPU: it builds, loads, exports every declared
symbol, and rejects bad input before touching the device."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from swe_fvm_gb300 import _lib, scenarios
from swe_fvm_gb300.solver import Fluxes, Wavespeeds, make_params, _swe_mesh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "swe_fvm_gb300.h")


def declared_symbols():
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(swe_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(_lib.EXPORTS) == syms


def test_header_compiles_as_c_and_cpp(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "swe_fvm_gb300.h"\nint main(void){swe_params p; return swe_params_default(&p);}\n')
    for comp, std in (("gcc", "-std=c99"), ("g++", "-std=c++17")):
        r = subprocess.run([comp, std, "-fsyntax-only", "-I", os.path.join(ROOT, "include"), "-x",
                            "c" if comp == "gcc" else "c++", str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_cpp_api_header_compiles():
    """The reference-named C++ layer: Fluxes::HLLC<Wavespeeds::Einfeldt> names
    a flux, SpaceDisc / TimeDisc / Solvers as in the reference."""
    src = ('#include "swe_fvm_gb300.hpp"\n'
           'static_assert(Fluxes::HLLC<Wavespeeds::Einfeldt>.flux == SWE_FLUX_HLLC, "");\n'
           'static_assert(Fluxes::HLL<Wavespeeds::Davis>.wavespeed == SWE_WS_DAVIS, "");\n'
           'void f(TimeDisc* td) { Solvers::SSPRK2(td, td->CFLdt()); }\n')
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                        os.path.join(ROOT, "include"), "-x", "c++", "-"], input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_params_default_are_the_reference_values():
    L = _lib.load()
    p = _lib.SweParams()
    assert L.swe_params_default(ctypes.byref(p)) == 0
    assert (p.flux, p.wavespeed, p.cor, p.tau, p.cfl) == (1, 2, 0.0, 0.0, 0.15)
    assert (p.reorder, p.block) == (-1, 0)  # device order and block sizes tuned


def _create(m, prim, fluxer=None):
    L = _lib.load()
    sm, keep = _swe_mesh(m)
    p = make_params(fluxer or Fluxes.HLLC(Wavespeeds.Einfeldt))
    ctx = ctypes.c_void_p()
    a = np.ascontiguousarray(prim, dtype=np.float64)
    st = L.swe_create(ctypes.byref(sm), a.ctypes.data, ctypes.byref(p), ctypes.byref(ctx))
    return st, L.swe_last_error(None).decode(), ctx


def _small():
    m, prim = scenarios.lake_at_rest(4)
    return m.contiguous(), prim


def test_rejects_non_wall_boundary_codes():
    """Only SOLID_WALL (-1) is implemented by the reference's flux loop."""
    m, prim = _small()
    ec = m.edge_cells.copy()
    ec[np.argmax(ec[:, 1] < 0), 1] = -2  # FREE_FLOW
    m.edge_cells = ec
    st, msg, _ = _create(m, prim)
    assert st == 2 and "-1" in msg


def test_rejects_out_of_range_and_inconsistent_topology():
    m, prim = _small()
    bad = m.contiguous()
    bad.cell_nodes = bad.cell_nodes.copy()
    bad.cell_nodes[0, 0] = 10 ** 6
    assert _create(bad, prim)[0] == 2
    bad = m.contiguous()
    bad.cell_neighbours = bad.cell_neighbours.copy()
    bad.cell_neighbours[5, 0] = 7 if bad.cell_neighbours[5, 0] != 7 else 8
    st, msg, _ = _create(bad, prim)
    assert st == 2 and "disagrees" in msg


def test_rejects_zero_area_cells():
    m, prim = _small()
    bad = m.contiguous()
    bad.geometry = bad.geometry.copy()
    a, b, c = bad.cell_nodes[0]
    bad.geometry[c, :2] = 0.5 * (bad.geometry[a, :2] + bad.geometry[b, :2])
    st, msg, _ = _create(bad, prim)
    assert st == 2 and "area" in msg


def test_rejects_null_arguments_and_bad_params():
    L = _lib.load()
    ctx = ctypes.c_void_p()
    assert L.swe_create(None, None, None, ctypes.byref(ctx)) == 1
    m, prim = _small()
    sm, keep = _swe_mesh(m)
    p = make_params(Fluxes.HLLC())
    p.flux = 7
    assert L.swe_create(ctypes.byref(sm), prim.ctypes.data, ctypes.byref(p), ctypes.byref(ctx)) == 1
    p = make_params(Fluxes.HLLC())
    p.cfl = -1.0
    assert L.swe_create(ctypes.byref(sm), prim.ctypes.data, ctypes.byref(p), ctypes.byref(ctx)) == 1
    assert L.swe_step(None, 1, 1e-3) == 1
    assert L.swe_destroy(None) == 1
    assert L.swe_last_error(None) is not None


def test_reference_module_name_imports():
    """``import SWE_FVM`` as with the reference's pybind module: Topology.create
    with its six arguments, copied (the reference's binding keeps references)."""
    import SWE_FVM

    m, _ = _small()
    args = [m.edge_nodes.copy(), m.edge_cells.copy(), m.cell_nodes.copy(), m.cell_edges.copy(),
            m.cell_neighbours.copy()]
    t = SWE_FVM.Topology.create(m.num_nodes, *args)
    for a in args:
        a[:] = -7  # the caller's arrays may change or go away
    assert t.num_elements() == m.num_cells and t.num_edges() == m.num_edges
    assert t.IsEdgeBoundary(int(np.argmax(m.edge_cells[:, 1] < 0)))
    for name in ("Domain", "SpaceDisc", "TimeDisc", "Solvers", "Fluxes", "Wavespeeds", "gauge_rollout"):
        assert hasattr(SWE_FVM, name)
