"""Device orders of cells, edges and nodes (swe_layout_plan, host only): each
strategy is a permutation with the documented structure, and the gather cost
model prefers a local order to a scattered one."""
import ctypes

import numpy as np
import pytest

from helpers import shuffle_mesh
from swe_fvm_gb300 import _lib, scenarios
from swe_fvm_gb300.mesh import build_topology, jittered_delaunay
from swe_fvm_gb300.solver import Fluxes, _swe_mesh, layout_plan, make_params


@pytest.fixture(scope="module")
def mesh():
    xyz, tri = jittered_delaunay(60, 3)
    return build_topology(xyz, tri).contiguous()


@pytest.fixture(scope="module")
def shuffled(mesh):
    return shuffle_mesh(mesh, 11)[0]


def _is_perm(p, n):
    return p.shape == (n,) and np.array_equal(np.sort(p), np.arange(n))


@pytest.mark.parametrize("strategy", ["keep", "morton", "rcm", "auto"])
def test_plans_are_permutations(shuffled, strategy):
    m = shuffled
    plan = layout_plan(m, strategy)
    assert _is_perm(plan["cell_from"], m.num_cells)
    assert _is_perm(plan["edge_from"], m.num_edges)
    assert _is_perm(plan["node_from"], m.num_nodes)
    if plan["chosen"] == "keep":
        assert np.array_equal(plan["cell_from"], np.arange(m.num_cells))


@pytest.mark.parametrize("strategy", ["morton", "rcm"])
def test_edges_follow_owners_and_nodes_first_cells(shuffled, strategy):
    m = shuffled
    plan = layout_plan(m, strategy)
    cf, ef, nf = plan["cell_from"], plan["edge_from"], plan["node_from"]
    cell_to = np.empty_like(cf)
    cell_to[cf] = np.arange(cf.size)
    owner_pos = cell_to[m.edge_cells[ef, 0]]
    assert np.all(np.diff(owner_pos) >= 0)
    node_to = np.empty_like(nf)
    node_to[nf] = np.arange(nf.size)
    first = np.full(m.num_nodes, m.num_cells)
    for j, i in enumerate(cf):
        for n in m.cell_nodes[i]:
            first[n] = min(first[n], j)
    assert np.all(np.diff(first[nf]) >= 0)


def test_morton_groups_nearby_centroids(shuffled):
    m = shuffled
    cen = m.centroids()[:, :2]

    def mean_step(order):
        return np.linalg.norm(np.diff(cen[order], axis=0), axis=1).mean()

    assert mean_step(layout_plan(m, "morton")["cell_from"]) < 0.2 * mean_step(np.arange(m.num_cells))


def test_rcm_narrows_the_neighbour_band(shuffled):
    m = shuffled
    cf = layout_plan(m, "rcm")["cell_from"]
    to = np.empty_like(cf)
    to[cf] = np.arange(cf.size)
    inner = m.edge_cells[:, 1] >= 0
    a, b = m.edge_cells[inner, 0], m.edge_cells[inner, 1]
    band_before = np.abs(a - b).max()
    band_after = np.abs(to[a] - to[b]).max()
    assert band_after < 0.1 * band_before
    assert band_after < 8 * np.sqrt(m.num_cells)


def test_auto_prefers_a_local_order(mesh, shuffled):
    shuf = layout_plan(shuffled, "auto")
    assert shuf["chosen"] in ("morton", "rcm")
    keep_cost, m_cost, r_cost = shuf["cost"]
    assert min(m_cost, r_cost) < 0.5 * keep_cost
    loc = layout_plan(mesh, "auto")
    c = dict(zip(("keep", "morton", "rcm"), loc["cost"]))
    assert c[loc["chosen"]] == min(c.values()) or loc["chosen"] == "keep"
    if loc["chosen"] != "keep":
        assert c[loc["chosen"]] < 0.95 * c["keep"]


def test_plan_is_deterministic(shuffled):
    a, b = layout_plan(shuffled, "auto"), layout_plan(shuffled, "auto")
    for k in ("cell_from", "edge_from", "node_from", "cost"):
        assert np.array_equal(a[k], b[k])


def test_disconnected_cells_are_all_placed():
    # two separate strips of triangles: RCM visits every component
    xyz, tri = jittered_delaunay(12, 5, morton=False)
    left = build_topology(xyz, tri)
    xyz2 = xyz.copy()
    xyz2[:, 0] += 3.0
    both = build_topology(np.vstack([xyz, xyz2]), np.vstack([tri, tri + xyz.shape[0]])).contiguous()
    plan = layout_plan(both, "rcm")
    assert _is_perm(plan["cell_from"], both.num_cells)
    half = left.num_cells
    side = plan["cell_from"] < half
    assert np.count_nonzero(np.diff(side.astype(int))) == 1  # one component after the other


def test_bad_reorder_and_block_are_rejected_before_the_device():
    L = _lib.load()
    m, prim = scenarios.lake_at_rest(4)
    m = m.contiguous()
    sm, keep = _swe_mesh(m)
    ctx = ctypes.c_void_p()
    for field, value in (("reorder", 3), ("reorder", -2), ("block", 48), ("block", 512), ("block", 16)):
        p = make_params(Fluxes.HLLC())
        setattr(p, field, value)
        assert L.swe_create(ctypes.byref(sm), prim.ctypes.data, ctypes.byref(p), ctypes.byref(ctx)) == 1, field
    assert L.swe_layout_plan(ctypes.byref(sm), 7, None, None, None, None, None) == 1


@pytest.mark.parametrize("strategy", ["morton", "rcm"])
def test_any_device_order_gives_the_restatement_the_same_bits(strategy):
    """The claim the device orders rest on, checked on the CPU restatement: the
    mesh renumbered by a plan (cells, edges, nodes; every row kept) steps to
    the same state, cell for cell, bit for bit."""
    from oracle.oracle import JACOBI, Oracle
    from swe_fvm_gb300.mesh import renumbered

    m, prim = scenarios.random_front_case(20, 6)
    m = m.contiguous()
    plan = layout_plan(m, strategy)
    cf = plan["cell_from"]
    r = renumbered(m, cf, plan["edge_from"], plan["node_from"])
    a = Oracle(m, prim, order=JACOBI)
    b = Oracle(r, prim[cf], order=JACOBI)
    for o in (a, b):
        o.compute_interface_values()
        o.compute_fluxes()
    for _ in range(6):
        dt = 0.15 * a.min_len_to_wavespeed()
        assert dt == 0.15 * b.min_len_to_wavespeed()
        a.step("SSPRK2", dt)
        b.step("SSPRK2", dt)
    assert np.array_equal(b.prim(), a.prim()[cf])
