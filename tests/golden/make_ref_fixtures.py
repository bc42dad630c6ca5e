"""Writes golden vectors produced by the reference's own solver.

The reference (NikitaMatckevich/SWE_FVM src/*.cpp, compiled into
oracle/_ref/libswe_ref.so by oracle/ref/build_ref.py with Q1 and Q20 patched)
runs each case below in jacobi loop order -- its own SpaceDisc / TimeDisc /
Fluxes / Solvers code, every TimeDisc::RHS of a stage taken before any cell is
written and every pass-2 reconstruction before any pass-2 write -- and the
states it reaches are stored in tests/golden/ref_<case>.npz together with the
mesh and the initial state (so nothing is regenerated on another machine,
where numpy's transcendental functions may round differently).  The GPU tests
(tests/test_gpu_ref_golden.py) replay each case through the library's public
API and compare bit for bit.

Needs the reference sources (it builds oracle/_ref first).
Usage: python tests/golden/make_ref_fixtures.py [case ...]
"""
from __future__ import annotations

import gzip
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.reference import JACOBI, Reference  # noqa: E402
from swe_fvm_gb300 import fileio, scenarios  # noqa: E402

PLUGINS = [(f, w) for f in ("HLL", "HLLC") for w in ("Rusanov", "Davis", "Einfeldt")]
SCHEMES = ("Euler", "SSPRK2", "SSPRK3")


def mesh_arrays(m):
    m = m.contiguous()
    return dict(geometry=m.geometry, edge_nodes=m.edge_nodes.astype(np.int32), edge_cells=m.edge_cells.astype(np.int32),
                cell_nodes=m.cell_nodes.astype(np.int32), cell_edges=m.cell_edges.astype(np.int32),
                cell_neighbours=m.cell_neighbours.astype(np.int32))


def bowl_mesh():
    """The reference's own examples/bowl.msh (tests/golden/bowl.msh.gz) with a
    flat bed, as examples/Main.cpp:172-180 sets it up."""
    import tempfile

    with gzip.open(os.path.join(HERE, "bowl.msh.gz"), "rb") as fh, tempfile.NamedTemporaryFile(suffix=".msh") as tmp:
        tmp.write(fh.read())
        tmp.flush()
        m = fileio.read_gmsh(tmp.name)
    m.geometry[:, 2] = 0.0
    return m


def run_cfl(m, prim, flux, ws, scheme, cfl, steps, snaps, cor=0.0):
    """dt = cfl x SpaceDisc::GetMinLenToWavespeed() of the latest flux pass
    before every step (the first from one ComputeInterfaceValues +
    ComputeFluxes of the initial state)."""
    r = Reference(m, prim, flux, ws, cor=cor, order=JACOBI)
    r.interface()
    out, t, dts = {}, 0.0, []
    for s in range(1, steps + 1):
        dt = cfl * r.min_len_to_wavespeed()
        r.step(scheme, dt)
        t += dt
        dts.append(dt)
        if s in snaps:
            out[f"prim_{s}"] = r.prim()
            out[f"t_{s}"] = np.float64(t)
    out["dts"] = np.array(dts)
    return out


def run_fixed(m, prim, flux, ws, scheme, dt, steps, snaps, cor=0.0):
    r = Reference(m, prim, flux, ws, cor=cor, order=JACOBI)
    out = {}
    for s in range(1, steps + 1):
        r.step(scheme, dt)
        if s in snaps:
            out[f"prim_{s}"] = r.prim()
    return out


def case_thacker64():
    """Workload: Thacker bowl, 64 x 64 x 2 = 8192 cells, HLLC + Einfeldt,
    SSPRK2, CFL 0.4, 1000 steps, walls."""
    m, prim = scenarios.thacker(64)
    res = run_cfl(m, prim, "HLLC", "Einfeldt", "SSPRK2", 0.4, 1000, (1, 10, 100, 1000))
    return dict(**mesh_arrays(m), prim0=prim, flux="HLLC", ws="Einfeldt", scheme="SSPRK2", cfl=0.4, steps=1000,
                snaps=np.array([1, 10, 100, 1000]), **res)


def case_bowl_gauss():
    """The reference's own driver case (examples/Main.cpp:172-195): bowl.msh,
    flat bed, w = 1 + exp(-5 r^2) about (4, 4), HLL + Einfeldt, Euler,
    dt = 1e-3; 20 steps.  The mesh is not stored: it is read again from
    tests/golden/bowl.msh.gz (text parsing is exact everywhere)."""
    m = bowl_mesh()
    prim = scenarios.gauss_wave(m)
    res = run_fixed(m, prim, "HLL", "Einfeldt", "Euler", 1e-3, 20, (20,))
    return dict(w0=prim[:, 0], flux="HLL", ws="Einfeldt", scheme="Euler", dt=1e-3, steps=20, snaps=np.array([20]),
                **res)


def case_dam_front():
    """Dam break over emerging bumps (the 1M-cell config's generator at
    lattice 40, 3k cells): wet/dry fronts; HLLC and HLL with Einfeldt,
    SSPRK2, CFL 0.15, 100 steps."""
    m, prim = scenarios.dam_break(lattice=40)
    out = dict(**mesh_arrays(m), prim0=prim, scheme="SSPRK2", cfl=0.15, steps=100, snaps=np.array([1, 10, 100]))
    for flux in ("HLLC", "HLL"):
        res = run_cfl(m, prim, flux, "Einfeldt", "SSPRK2", 0.15, 100, (1, 10, 100))
        out.update({f"{flux}_{k}": v for k, v in res.items()})
    return out


def case_front_plugins():
    """Every flux x wave-speed plugin and every scheme on the small wet/dry
    front mesh (all reconstruction branches), dt = 2e-3, 6 steps; the
    interface values, fluxes, node maxima and CFL ratio of the initial state
    (HLLC + Einfeldt); Coriolis 0.7 with SSPRK3 over 5 steps."""
    m, prim = scenarios.random_front_case(16, seed=2)
    out = dict(**mesh_arrays(m), prim0=prim, dt=2e-3, steps=6)
    for f, w in PLUGINS:
        for s in SCHEMES:
            out[f"{f}_{w}_{s}"] = run_fixed(m, prim, f, w, s, 2e-3, 6, (6,))["prim_6"]
    r = Reference(m, prim, "HLLC", "Einfeldt", order=JACOBI)
    r.interface()
    edg, src, f, mx = r.edge_fields()
    out.update(edg=edg, src=src[:, 1:], fluxes=f, max_wp=mx, ratio=np.float64(r.min_len_to_wavespeed()),
               classes=r.classify())
    out["coriolis_SSPRK3"] = run_fixed(m, prim, "HLLC", "Einfeldt", "SSPRK3", 2e-3, 5, (5,), cor=0.7)["prim_5"]
    return out


CASES = {"thacker64": case_thacker64, "bowl_gauss": case_bowl_gauss, "dam_front": case_dam_front,
         "front_plugins": case_front_plugins}


def main(names):
    for name in names or CASES:
        t0 = time.time()
        data = CASES[name]()
        dst = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(dst, **{k: np.asarray(v) for k, v in data.items()})
        print(f"{dst}: {os.path.getsize(dst)} bytes, {time.time() - t0:.1f} s")


if __name__ == "__main__":
    main(sys.argv[1:])
