"""Device integrals (volume, kinetic and potential energy), a Gmsh-read mesh
through the GPU step, and the analytic layer driving a run."""
import math

import numpy as np
import pytest

from oracle.oracle import Oracle
from swe_fvm_gb300 import (Batch, Fluxes, Solvers, SpaceDisc, TimeDisc, Wavespeeds, analytic, diagnostics, fileio,
                           scenarios)
from swe_fvm_gb300.mesh import structured_square

pytestmark = pytest.mark.gpu


def host_integrals(mesh, prim):
    b = mesh.centroids()[:, 2]
    h = prim[:, 0] - b
    wet = h > 1e-12
    A = mesh.areas()
    u, v = prim[:, 1], prim[:, 2]
    return np.array([A[wet] @ h[wet], A[wet] @ (0.5 * h[wet] * (u[wet] ** 2 + v[wet] ** 2)),
                     A[wet] @ (0.5 * h[wet] ** 2 + h[wet] * b[wet])])


def test_integrals_match_host_sums_and_volume_is_conserved(gpu):
    m, prim = scenarios.random_front_case(24, 2)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    ints0 = sd.integrals()
    assert np.allclose(ints0, host_integrals(m, sd.GetVolField()), rtol=1e-13, atol=1e-15)
    assert np.array_equal(ints0, sd.integrals())  # deterministic
    sd.run_cfl(1, 50)
    ints1 = sd.integrals()
    assert np.allclose(ints1, host_integrals(m, sd.GetVolField()), rtol=1e-13, atol=1e-15)
    assert ints1[0] == pytest.approx(ints0[0], rel=1e-12)  # walls: the volume stays


def test_batch_integrals_equal_single(gpu):
    cases = [scenarios.random_front_case(16, s) for s in (1, 2)]
    b = Batch([c[0] for c in cases], [c[1] for c in cases])
    b.run_cfl(1, 10)
    for q, (m, p) in enumerate(cases):
        sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p)
        sd.run_cfl(1, 10)
        assert np.array_equal(b.integrals(q), sd.integrals())


def test_gmsh_mesh_runs_bit_exact_against_the_oracle(gpu, tmp_path):
    """A mesh read from an ASCII Gmsh file drives the GPU step; 5 SSPRK2 steps
    equal the CPU restatement's."""
    sol = analytic.ClassicThacker(0.1, math.sqrt(0.3))
    base = structured_square(12, -2.0, 2.0, bathymetry=sol.b)
    xyz, tri = base.geometry, base.cell_nodes
    lines = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Nodes", f"1 {len(xyz)} 1 {len(xyz)}",
             f"2 1 0 {len(xyz)}"]
    lines += [str(k + 1) for k in range(len(xyz))]
    lines += [f"{float(x)!r} {float(y)!r} {float(z)!r}" for x, y, z in xyz]
    lines += ["$EndNodes", "$Elements", f"1 {len(tri)} 1 {len(tri)}", f"2 1 2 {len(tri)}"]
    lines += [f"{k + 1} {a + 1} {b + 1} {c + 1}" for k, (a, b, c) in enumerate(tri)]
    lines.append("$EndElements")
    p = tmp_path / "bowl.msh"
    p.write_text("\n".join(lines) + "\n")
    m = fileio.read_gmsh(str(p))
    prim = analytic.initial_state(m, sol, 0.0, n=10)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    td = TimeDisc(sd)
    o = Oracle(m, prim)
    dt = 2e-3
    for _ in range(5):
        Solvers.SSPRK2(td, dt)
        o.step("SSPRK2", dt)
    assert np.array_equal(sd.GetVolField(), o.prim())
    # the L2 error of the depth against the closed form at t = 5 dt stays a
    # small fraction of the depth's own L2 norm on this coarse mesh
    exact = analytic.cell_averages(m, sol, 5 * dt, n=6)
    e1 = diagnostics.l2_errors(m, sd.GetVolField(), sol, 5 * dt, n=6)
    assert np.all(np.isfinite(e1))
    assert e1[0] < 0.02 * np.sqrt(m.areas() @ exact[:, 0] ** 2)
