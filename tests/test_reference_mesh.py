"""The library's Gmsh reader on the reference's own mesh file.

tests/golden/bowl.msh.gz is the reference's examples/bowl.msh (Gmsh 4.1,
7555 nodes); tests/golden/bowl_euler.npz holds the topology the reference
wrote for it (notebooks/topology.dat, examples/Main.cpp:146-165) and its node
coordinates (notebooks/geometry.dat, 6 significant digits).  Integer work is
pinned exactly, under one stated canonical renumbering: edges are matched by
their (unordered) node pair, because the reference's older reader numbered
the boundary edges first.  Then
  * cell -> nodes and cell -> neighbours are identical, row for row;
  * cell -> edges is identical position for position (edge k of a cell joins
    its nodes k and k+1, the neighbour k lies across it);
  * edge -> cells is identical as an unordered pair, with -1 (SOLID_WALL) in
    column 1 for every boundary edge in both (which cell owns an interior
    edge, column 0, may differ: the flux sign follows the owner).
"""
import os

import numpy as np

from tests.helpers import GOLDEN, read_bowl_mesh


def test_gmsh_reader_reproduces_reference_topology():
    m = read_bowl_mesh()
    d = np.load(os.path.join(GOLDEN, "bowl_euler.npz"))
    geo, ed, cd = d["geometry"], d["edges"].astype(np.int64), d["cells"].astype(np.int64)
    assert (m.num_nodes, m.num_edges, m.num_cells) == (7555, 22342, 14788)
    assert geo.shape[0] == m.num_nodes and ed.shape[0] == m.num_edges and cd.shape[0] == m.num_cells
    # coordinates: the dump printed 6 significant digits of values in [0, 8]
    assert np.max(np.abs(m.geometry[:, :2] - geo[:, :2])) < 1e-5
    assert np.array_equal(m.cell_nodes, cd[:, :3])
    assert np.array_equal(m.cell_neighbours, cd[:, 6:])

    def key(en):
        return np.minimum(en[:, 0], en[:, 1]) * m.num_nodes + np.maximum(en[:, 0], en[:, 1])

    ours = {int(k): i for i, k in enumerate(key(m.edge_nodes))}
    assert len(ours) == m.num_edges
    match = np.array([ours[int(k)] for k in key(ed[:, :2])])  # reference edge -> our edge
    assert len(np.unique(match)) == m.num_edges
    assert np.array_equal(match[cd[:, 3:6]], m.cell_edges)
    ec_ref, ec_ours = ed[:, 2:], m.edge_cells[match]
    assert np.array_equal(np.sort(ec_ref, axis=1), np.sort(ec_ours, axis=1))
    walls_ref, walls_ours = ec_ref[:, 1] < 0, ec_ours[:, 1] < 0
    assert np.array_equal(walls_ref, walls_ours) and walls_ref.sum() == 320
    assert np.all(ec_ref[walls_ref, 1] == -1) and np.all(ec_ours[walls_ours, 1] == -1)
    # every boundary edge is owned by its one cell in both
    assert np.array_equal(ec_ref[walls_ref, 0], ec_ours[walls_ours, 0])
