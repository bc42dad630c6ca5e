"""Mesh ingestion (Gmsh 2.2 / 4.1, ASCII and binary), the reference's text outputs, and the
closed-form solutions of the test layer (CPU only)."""
import math

import numpy as np
import pytest

from swe_fvm_gb300 import analytic, diagnostics, fileio, scenarios
from swe_fvm_gb300.mesh import build_topology, structured_square


def _grid(n=4):
    m = structured_square(n, 0.0, 1.0)
    return m.geometry, m.cell_nodes


def _write_gmsh41(path, xyz, tri, extra_node=True):
    # one surface block of nodes (+ an unused node in a point block), a block
    # of boundary lines and a block of triangles; tags start at 1
    n = len(xyz)
    lines = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$Nodes"]
    blocks = 2 if extra_node else 1
    total = n + (1 if extra_node else 0)
    lines.append(f"{blocks} {total} 1 {total}")
    lines.append(f"2 1 0 {n}")
    lines += [str(k + 1) for k in range(n)]
    lines += [f"{float(x)!r} {float(y)!r} {float(z)!r}" for x, y, z in xyz]
    if extra_node:
        lines += ["0 7 0 1", str(n + 1), "9.0 9.0 0.0"]
    lines.append("$EndNodes")
    lines.append("$Elements")
    lines.append(f"2 {1 + len(tri)} 1 {1 + len(tri)}")
    lines += ["1 3 1 1", "1 1 2"]
    lines.append(f"2 1 2 {len(tri)}")
    lines += [f"{k + 2} {a + 1} {b + 1} {c + 1}" for k, (a, b, c) in enumerate(tri)]
    lines.append("$EndElements")
    path.write_text("\n".join(lines) + "\n")


def _write_gmsh22(path, xyz, tri):
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(len(xyz))]
    lines += [f"{k + 10} {float(x)!r} {float(y)!r} {float(z)!r}" for k, (x, y, z) in enumerate(xyz)]
    lines += ["$EndNodes", "$Elements", str(len(tri) + 1), "1 1 2 0 1 10 11"]
    lines += [f"{k + 2} 2 2 0 1 {a + 10} {b + 10} {c + 10}" for k, (a, b, c) in enumerate(tri)]
    lines.append("$EndElements")
    path.write_text("\n".join(lines) + "\n")


def _same_mesh(a, b):
    for name in ("geometry", "edge_nodes", "edge_cells", "cell_nodes", "cell_edges", "cell_neighbours"):
        assert np.array_equal(getattr(a, name), getattr(b, name)), name


@pytest.mark.parametrize("fmt", ["4.1", "2.2"])
def test_read_gmsh_builds_the_reference_topology(tmp_path, fmt):
    xyz, tri = _grid(5)
    xyz = xyz.copy()
    xyz[:, 2] = 0.1 * xyz[:, 0] - 0.05 * xyz[:, 1]
    p = tmp_path / "m.msh"
    (_write_gmsh41 if fmt == "4.1" else _write_gmsh22)(p, xyz, tri)
    m = fileio.read_gmsh(str(p))
    _same_mesh(m, build_topology(xyz, tri))
    # walls: edges with one cell; every neighbour relation is symmetric
    walls = m.edge_cells[:, 1] < 0
    assert walls.sum() == 4 * 5
    for c in range(m.num_cells):
        for k in range(3):
            nb = m.cell_neighbours[c, k]
            if nb >= 0:
                assert c in m.cell_neighbours[nb]


def test_read_gmsh_bathymetry_override(tmp_path):
    xyz, tri = _grid(3)
    p = tmp_path / "m.msh"
    _write_gmsh41(p, xyz, tri)
    m = fileio.read_gmsh(str(p), bathymetry=lambda x, y: x * y)
    assert np.allclose(m.geometry[:, 2], m.geometry[:, 0] * m.geometry[:, 1])


@pytest.mark.parametrize("version", ["4.1", "2.2"])
@pytest.mark.parametrize("binary", [False, True])
def test_write_and_read_gmsh_round_trip(tmp_path, version, binary):
    m = structured_square(7, 0.0, 2.0, bathymetry=lambda x, y: 0.1 * x - 0.2 * y * y)
    p = tmp_path / "m.msh"
    fileio.write_gmsh(str(p), m, version, binary)
    _same_mesh(fileio.read_gmsh(str(p)), m.contiguous())


def _write_gmsh41_binary(path, xyz, tri, endian="<"):
    # a point block with an unused node, a surface node block, a line block
    # and a triangle block, like a file Gmsh writes for a 2-D model
    u8, i4, f8 = endian + "u8", endian + "i4", endian + "f8"
    n = len(xyz)
    parts = [b"$MeshFormat\n4.1 1 8\n", np.array([1], i4).tobytes(), b"\n$EndMeshFormat\n$Nodes\n"]
    parts += [np.array([2, n + 1, 1, n + 1], u8).tobytes()]
    parts += [np.array([0, 7, 0], i4).tobytes(), np.array([1, n + 1], u8).tobytes(),
              np.array([9.0, 9.0, 0.0], f8).tobytes()]
    parts += [np.array([2, 1, 0], i4).tobytes(), np.array([n], u8).tobytes(),
              np.arange(1, n + 1, dtype=u8).tobytes(), np.asarray(xyz, f8).tobytes()]
    parts += [b"\n$EndNodes\n$Elements\n", np.array([2, len(tri) + 1, 1, len(tri) + 1], u8).tobytes()]
    parts += [np.array([1, 3, 1], i4).tobytes(), np.array([1], u8).tobytes(), np.array([1, 1, 2], u8).tobytes()]
    ids = np.arange(2, len(tri) + 2)
    parts += [np.array([2, 1, 2], i4).tobytes(), np.array([len(tri)], u8).tobytes(),
              np.column_stack([ids, np.asarray(tri) + 1]).astype(u8).tobytes(), b"\n$EndElements\n"]
    path.write_bytes(b"".join(parts))


@pytest.mark.parametrize("endian", ["<", ">"])
def test_read_binary_gmsh41_with_other_blocks(tmp_path, endian):
    xyz, tri = _grid(5)
    p = tmp_path / "b.msh"
    _write_gmsh41_binary(p, xyz, tri, endian)
    _same_mesh(fileio.read_gmsh(str(p)), build_topology(xyz, tri))


def _write_gmsh22_binary(path, xyz, tri, nl=b"\n"):
    # what Gmsh writes for a 2-D model: a point block (type 15) and a line
    # block (type 1) with 2 tags each before the triangles; `nl` ends the text
    # lines (LF or CRLF)
    n, c = len(xyz), len(tri)
    parts = [b"$MeshFormat" + nl + b"2.2 1 8" + nl, np.array([1], "<i4").tobytes(), nl + b"$EndMeshFormat" + nl]
    parts += [b"$Nodes" + nl + str(n).encode() + nl]
    rec = np.zeros(n, np.dtype([("tag", "<i4"), ("xyz", "<f8", (3,))]))
    rec["tag"] = np.arange(1, n + 1)
    rec["xyz"] = xyz
    parts += [rec.tobytes(), nl + b"$EndNodes" + nl + b"$Elements" + nl + str(c + 3).encode() + nl]
    parts += [np.array([15, 1, 2], "<i4").tobytes(), np.array([1, 7, 7, 1], "<i4").tobytes()]
    parts += [np.array([1, 2, 2], "<i4").tobytes(), np.array([[2, 3, 3, 1, 2], [3, 3, 3, 2, 3]], "<i4").tobytes()]
    ids = np.arange(4, c + 4)
    rows = np.column_stack([ids, np.full(c, 5), np.full(c, 5), np.asarray(tri) + 1]).astype("<i4")
    parts += [np.array([2, c, 2], "<i4").tobytes(), rows.tobytes(), nl + b"$EndElements" + nl]
    path.write_bytes(b"".join(parts))


@pytest.mark.parametrize("nl", [b"\n", b"\r\n"], ids=["lf", "crlf"])
def test_read_binary_gmsh22_with_point_and_line_blocks(tmp_path, nl):
    xyz, tri = _grid(5)
    p = tmp_path / "b22.msh"
    _write_gmsh22_binary(p, xyz, tri, nl)
    _same_mesh(fileio.read_gmsh(str(p)), build_topology(xyz, tri))


def test_read_binary_gmsh41_crlf_headers(tmp_path):
    xyz, tri = _grid(4)
    p = tmp_path / "b.msh"
    _write_gmsh41_binary(p, xyz, tri)
    data = p.read_bytes()
    for key in (b"$MeshFormat\n", b"$EndMeshFormat\n", b"$Nodes\n", b"$EndNodes\n", b"$Elements\n"):
        data = data.replace(key, key[:-1] + b"\r\n", 1)
    p.write_bytes(data)
    _same_mesh(fileio.read_gmsh(str(p)), build_topology(xyz, tri))


def test_read_gmsh_rejects_truncated_binary(tmp_path):
    xyz, tri = _grid(4)
    p = tmp_path / "b.msh"
    _write_gmsh41_binary(p, xyz, tri)
    p.write_bytes(p.read_bytes()[:-200])
    with pytest.raises(ValueError):
        fileio.read_gmsh(str(p))
    p.write_text("$MeshFormat\n3.0 0 8\n$EndMeshFormat\n")
    with pytest.raises(ValueError):
        fileio.read_gmsh(str(p))


def test_dump_domain_round_trip_and_fields(tmp_path):
    m = structured_square(6, -1.0, 1.0, bathymetry=lambda x, y: 0.1 * (x * x + y * y))
    g, t = tmp_path / "geometry.dat", tmp_path / "topology.dat"
    fileio.dump_domain(m, str(g), str(t))
    _same_mesh(fileio.load_domain(str(g), str(t)), m)
    prim = np.zeros((m.num_cells, 3))
    prim[:, 0] = m.centroids()[:, 2] + 0.3
    prim[:, 1], prim[:, 2] = 0.5, -0.25
    f = tmp_path / "fields.dat"
    fileio.dump_fields(m, prim, str(f))
    rows = np.loadtxt(f)
    assert rows.shape == (m.num_cells, 3)
    assert np.allclose(rows[:, 0], prim[:, 0])
    assert np.allclose(rows[:, 1], 0.3 * 0.5) and np.allclose(rows[:, 2], 0.3 * -0.25)


SOLUTIONS = {
    "ball": analytic.Ball(0.1, 0.3, -0.2, 0.05, 0.02, cor=0.2),
    "conservative_thacker": analytic.ConservativeThacker(0.1, 0.5, 0.05, 0.02, cor=0.1),
    "solenoidal_thacker": analytic.SolenoidalThacker(0.1, 0.5, 0.0, 0.3),
    "classic_thacker": analytic.ClassicThacker(0.1, math.sqrt(0.3)),
    "classic_thacker_rotating": analytic.ClassicThacker(0.1, math.sqrt(0.3), 0.02, 0.1, cor=0.2),
}


@pytest.mark.parametrize("name", list(SOLUTIONS))
def test_closed_forms_solve_the_shallow_water_equations(name):
    """Central differences of mass and momentum (g = 1, Coriolis source
    cor (v, -u)) vanish at wet points to round-off."""
    s = SOLUTIONS[name]
    rng = np.random.default_rng(3)
    x, y, t, d = rng.uniform(-0.4, 0.4, 300), rng.uniform(-0.4, 0.4, 300), 0.7, 1e-5
    wet = s.h(x, y, t) > 1e-3
    x, y = x[wet], y[wet]
    D = lambda f, dx, dy, dt: (f(x + dx, y + dy, t + dt) - f(x - dx, y - dy, t - dt)) / (2 * d)
    mass = D(s.h, 0, 0, d) + D(s.hu, d, 0, 0) + D(s.hv, 0, d, 0)
    u, v = s.u(x, y, t), s.v(x, y, t)
    mx = D(s.u, 0, 0, d) + u * D(s.u, d, 0, 0) + v * D(s.u, 0, d, 0) + D(s.w, d, 0, 0) - s.cor * v
    my = D(s.v, 0, 0, d) + u * D(s.v, d, 0, 0) + v * D(s.v, 0, d, 0) + D(s.w, 0, d, 0) + s.cor * u
    assert wet.sum() > 100
    assert max(np.abs(mass).max(), np.abs(mx).max(), np.abs(my).max()) < 1e-8


def test_ball_starts_at_its_initial_position_and_velocity():
    b = analytic.Ball(0.1, 0.3, -0.2, 0.05, 0.02, cor=0.2)
    phim, phip, psim, psip = b._modes(0.0)
    assert (phim + phip, psim + psip) == pytest.approx((0.3, -0.2), abs=1e-14)
    assert b._velocity(0.0) == pytest.approx((0.05, 0.02), abs=1e-14)


def test_classic_thacker_matches_the_config_restatement():
    from swe_fvm_gb300.scenarios import ClassicThacker as ConfigThacker

    a, c = analytic.ClassicThacker(0.1, math.sqrt(0.3)), ConfigThacker()
    rng = np.random.default_rng(4)
    x, y = rng.uniform(-2, 2, 100), rng.uniform(-2, 2, 100)
    for t in (0.0, 0.9, 3.1):
        assert np.allclose(a.h(x, y, t), c.h(x, y, t), atol=1e-14)
        assert np.allclose(a.u(x, y, t), c.u(x, y, t), atol=1e-14)
        assert np.allclose(a.v(x, y, t), c.v(x, y, t), atol=1e-14)
    assert np.allclose(a.b(x, y) + 0.1, c.bed(x, y))  # the config bowl is shifted by +delta


def test_initial_state_and_l2_error_of_exact_averages():
    s = analytic.ClassicThacker(0.1, math.sqrt(0.3))
    m = structured_square(16, -2.0, 2.0, bathymetry=s.b)
    prim = analytic.initial_state(m, s, 0.0, n=8)
    # the volume of the averages is the exact volume of the paraboloid cap
    vol = m.areas() @ (prim[:, 0] - m.centroids()[:, 2])
    assert vol > 0
    # lake at rest: zero velocity, flat surface where wet
    lr = analytic.LakeAtRest()
    ml = structured_square(8, 0.0, 4.0, bathymetry=lr.b)
    pl = analytic.initial_state(ml, lr, 0.0, n=4)
    assert np.all(pl[:, 1:] == 0.0)
    # l2 error of a state built from the same averages: zero
    avg = analytic.cell_averages(m, s, 0.0, n=8)
    p = np.zeros_like(avg)
    p[:, 0] = avg[:, 0] + m.centroids()[:, 2]
    wet = avg[:, 0] > 0
    p[wet, 1] = avg[wet, 1] / avg[wet, 0]
    p[wet, 2] = avg[wet, 2] / avg[wet, 0]
    assert np.all(diagnostics.l2_errors(m, p, s, 0.0, n=8) < 1e-13)


def test_checkpoint_round_trip_is_bitwise_and_mesh_bound(tmp_path):
    from swe_fvm_gb300.fileio import load_state, save_state

    m, prim = scenarios.random_front_case(10, 1)
    prim = prim + np.random.default_rng(0).normal(0, 1e-9, prim.shape)
    save_state(str(tmp_path / "ck.npz"), m, prim, t=0.123456789, step=42, cfl_ratio=0.0123)
    p2, t, step, r = load_state(str(tmp_path / "ck.npz"), m)
    assert np.array_equal(p2.view(np.uint64), prim.view(np.uint64))
    assert (t, step, r) == (0.123456789, 42, 0.0123)
    other, _ = scenarios.random_front_case(10, 2)
    with pytest.raises(ValueError):
        load_state(str(tmp_path / "ck.npz"), other)


def test_read_gmsh_rejects_an_undefined_node_tag(tmp_path):
    xyz, tri = _grid(3)
    tri = tri.copy()
    tri[0, 1] = len(xyz) + 40  # no such node
    p = tmp_path / "m.msh"
    _write_gmsh22(p, xyz, tri)
    with pytest.raises(ValueError, match="node tag"):
        fileio.read_gmsh(str(p))
