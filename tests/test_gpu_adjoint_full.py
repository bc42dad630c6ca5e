"""The discrete adjoint against central finite differences at the adjoint
benchmark configurations' full sizes.

The 250k-cell run: one 250k-cell instance, 2000 SSPRK2 steps, 64 gauge cells observed
every 10th step, checkpoint every 50 steps, target traces from a run whose bed
carries 5 % seeded Gaussian noise; gradient with respect to the initial
surface, central differences at step 1e-6 on 32 cells drawn at random from the
wet cells (h > 0.02).
The 64-instance batch: 64 instances of 20k-100k cells, 500 steps, 16 gauges each,
checkpoint every 25 steps, the same kind of target; gradient with respect to
the node bathymetry, central differences at step 1e-6 on 12 nodes per instance
drawn at random from the interior nodes whose cells are all wet, every
instance perturbed in the same batched run.

Every perturbed run repeats the taped run's dts (swe_run_traces), so the
differences see the same discrete map the adjoint differentiates.

Admissibility, stated before any difference is compared:
  * resolvable: |gradient| >= 1e-3 of the largest over the candidates (in
    the batch, over the instance's own candidates) and neither difference
    exactly zero; in the batch also |gradient| >= 1e-6 per unit of bed height.
    That floor was added after a run in which five nodes far from every gauge,
    with gradients of 7e-9 to 5e-7, disagreed by 1.6e-6 to 3e-3 while their
    differences had converged: such gradients are sums dominated by
    cancellation, at the round-off level of both the forward and the reverse;
  * converged: the central differences at eps and eps / 2 agree to 1e-6
    relative.  A limiter, wet/dry or upwind switch inside the stencil makes
    them disagree (a jump J moves each by ~J / eps), so this certifies that
    the loss is smooth at the scale of the step;
  * not regularised: the gradient with the wetting-front regularisation of the
    reverse (swe_adjoint_set_regularisation, depth 1e-3, the default) equals
    the exact one (depth 0) to 1e-7 relative.
  * the batch only, a condition on the candidates: the bed around the node
    (its cells' nodes and their neighbours' nodes) has a relief of at least
    1000 eps.  Where the bed is flatter than the step (parts of these floors
    are flat to 1e-10), the binary limiter's decisions in the stencil compare
    offsets smaller than the step, so every perturbed run takes another branch
    and the differences converge to that branch's slope, not to the
    derivative at the unperturbed bed.
On every admissible cell or node the adjoint must agree with the differences
to 1e-6 relative (the target bound, nothing relaxed); every resolvable and
converged cell of the 250k-cell run must also agree with the exact (unregularised)
gradient to 1e-6.  The test prints the whole error distribution.
"""
import numpy as np
import pytest

from swe_fvm_gb300 import scenarios
from swe_fvm_gb300.adjoint import BatchRollout, Rollout
from swe_fvm_gb300.mesh import Mesh

pytestmark = pytest.mark.gpu

EPS = 1e-6
BOUND = 1e-6


def with_bed(m, z):
    g = m.geometry.copy()
    g[:, 2] = z
    return Mesh(g, m.edge_nodes, m.edge_cells, m.cell_nodes, m.cell_edges, m.cell_neighbours)


def bed_relief(m):
    """max - min of the bed over each node's cells' nodes and their
    neighbours' nodes."""
    z = m.geometry[:, 2]
    cz_max = z[m.cell_nodes].max(axis=1)
    cz_min = z[m.cell_nodes].min(axis=1)
    nb = m.cell_neighbours
    ring_max = np.where(nb >= 0, cz_max[np.maximum(nb, 0)], -np.inf).max(axis=1)
    ring_min = np.where(nb >= 0, cz_min[np.maximum(nb, 0)], np.inf).min(axis=1)
    ring_max = np.maximum(ring_max, cz_max)
    ring_min = np.minimum(ring_min, cz_min)
    hi = np.full(m.num_nodes, -np.inf)
    lo = np.full(m.num_nodes, np.inf)
    np.maximum.at(hi, m.cell_nodes.reshape(-1), np.repeat(ring_max, 3))
    np.minimum.at(lo, m.cell_nodes.reshape(-1), np.repeat(ring_min, 3))
    return hi - lo


def summary(name, rows):
    rel = np.array([r["rel"] for r in rows])
    adm = np.array([r["admissible"] for r in rows])
    print(f"\n{name}: {len(rows)} tested, {adm.sum()} admissible; relative error on admissible: "
          f"median {np.median(rel[adm]) if adm.any() else float('nan'):.2e}, "
          f"max {rel[adm].max() if adm.any() else float('nan'):.2e}; all tested: median {np.median(rel):.2e}")
    for r in sorted(rows, key=lambda r: r["rel"]):
        print("   ", {k: (f"{v:.3e}" if isinstance(v, float) else v) for k, v in r.items()})


def test_adjoint_250k_initial_surface_gradient_central_differences(gpu):
    steps, obs, ckpt = 2000, 10, 50
    mesh, prim = scenarios.hump_instance(2024, 250000)
    mesh = mesh.contiguous()
    gauges = np.random.default_rng(11).choice(mesh.num_cells, 64, replace=False)
    zt = mesh.geometry[:, 2] * (1 + 0.05 * np.random.default_rng(12).normal(size=mesh.num_nodes))
    target = Rollout(with_bed(mesh, zt), prim).forward(1, steps, ckpt, gauges, obs)
    ro = Rollout(mesh, prim)
    tr = ro.forward(1, steps, ckpt, gauges, obs)
    dts = ro.dts(steps)
    g_reg = ro.backward(2.0 * (tr - target))[0][:, 0]
    ro.set_regularisation(0.0)
    g_ex = ro.backward(2.0 * (tr - target))[0][:, 0]
    ro.set_regularisation(1e-3)
    sd = ro.sd

    def loss(p):
        sd.SetVolField(p)
        return float(np.sum((sd.run_traces(1, dts, gauges, obs) - target) ** 2))

    assert loss(prim) == float(np.sum((tr - target) ** 2))  # the trace run repeats the taped run
    wet = np.where(prim[:, 0] - mesh.centroids()[:, 2] > 0.02)[0]
    gmax = np.abs(g_reg[wet]).max()
    rows = []
    for c in np.random.default_rng(99).choice(wet, 32, replace=False):
        fd = []
        for e in (EPS, EPS / 2):
            v = []
            for s in (1.0, -1.0):
                p = prim.copy()
                p[c, 0] += s * e
                v.append(loss(p))
            fd.append((v[0] - v[1]) / (2 * e))
        resolvable = abs(g_reg[c]) >= 1e-3 * gmax and fd[0] != 0.0 and fd[1] != 0.0
        converged = abs(fd[0] - fd[1]) <= 1e-6 * abs(fd[1])
        unreg = abs(g_reg[c] - g_ex[c]) <= 1e-7 * abs(g_ex[c])
        rows.append({"cell": int(c), "adjoint": float(g_reg[c]), "fd": fd[0],
                     "rel": abs(g_reg[c] - fd[0]) / max(abs(fd[0]), 1e-300),
                     "rel_exact": abs(g_ex[c] - fd[0]) / max(abs(fd[0]), 1e-300),
                     "resolvable": bool(resolvable), "converged": bool(converged), "unregularised": bool(unreg),
                     "admissible": bool(resolvable and converged and unreg)})
    summary("250k cells, 2000 steps", rows)
    adm = [r for r in rows if r["admissible"]]
    assert len(adm) >= 8
    assert max(r["rel"] for r in adm) <= BOUND
    rc = [r for r in rows if r["resolvable"] and r["converged"]]
    assert max(r["rel_exact"] for r in rc) <= BOUND


def test_batched_adjoint_64_instances_bathymetry_gradient_central_differences(gpu):
    steps, obs, ckpt, K = 500, 10, 25, 12
    ens = scenarios.adjoint_ensemble(64)
    meshes = [e[0].contiguous() for e in ens]
    prims = [e[1] for e in ens]
    NI = len(meshes)
    gauges = [np.random.default_rng(300 + q).choice(m.num_cells, 16, replace=False) for q, m in enumerate(meshes)]
    rng = np.random.default_rng(7)
    zt = [m.geometry[:, 2] * (1 + 0.05 * rng.normal(size=m.num_nodes)) for m in meshes]
    z0 = [m.geometry[:, 2].copy() for m in meshes]
    br = BatchRollout(meshes, prims, cfl=0.4)
    b = br.batch
    b.set_bathymetry(zt)
    b.prime()
    target = br.forward(1, steps, ckpt, gauges, obs)
    b.set_bathymetry(z0)
    for q in range(NI):
        b.set_prim(q, prims[q])
    b.prime()
    tr = br.forward(1, steps, ckpt, gauges, obs)
    dts = br.dts(steps)
    tg = [2.0 * (t - tt) for t, tt in zip(tr, target)]
    g_reg = [g[1] for g in br.backward(tg)]
    br.set_regularisation(0.0)
    g_ex = [g[1] for g in br.backward(tg)]
    br.set_regularisation(1e-3)
    coff = br.cell_off
    gcat = np.concatenate([g + coff[q] for q, g in enumerate(gauges)])
    cut = np.cumsum([0] + [len(g) for g in gauges])

    def losses(zs):
        b.set_bathymetry(zs)
        for q in range(NI):
            b.set_prim(q, prims[q])
        out = b.run_traces(1, dts, gcat, obs)
        return np.array([np.sum((out[:, cut[q]:cut[q + 1]] - target[q]) ** 2) for q in range(NI)])

    picks, cands = [], []
    for q, m in enumerate(meshes):
        h = prims[q][:, 0] - m.centroids()[:, 2]
        nmin = np.full(m.num_nodes, np.inf)
        np.minimum.at(nmin, m.cell_nodes.reshape(-1), np.repeat(h, 3))
        bnd = np.zeros(m.num_nodes, bool)
        bnd[m.edge_nodes[m.edge_cells[:, 1] < 0].reshape(-1)] = True
        relief = bed_relief(m)
        cand = np.where((nmin > 0.02) & ~bnd & (relief >= 1e3 * EPS))[0]
        cands.append(cand)
        picks.append(np.random.default_rng(500 + q).choice(cand, K, replace=False) if len(cand) >= K else None)
    rows = []
    for k in range(K):
        fd = []
        for e in (EPS, EPS / 2):
            v = []
            for s in (1.0, -1.0):
                zs = []
                for q in range(NI):
                    z = z0[q].copy()
                    if picks[q] is not None:
                        z[picks[q][k]] += s * e
                    zs.append(z)
                v.append(losses(zs))
            fd.append((v[0] - v[1]) / (2 * e))
        for q in range(NI):
            if picks[q] is None:
                continue
            nd = picks[q][k]
            gmax = np.abs(g_reg[q][cands[q]]).max()
            gr, ge, f0, f1 = g_reg[q][nd], g_ex[q][nd], fd[0][q], fd[1][q]
            resolvable = bool(gmax > 0 and abs(gr) >= max(1e-3 * gmax, 1e-6) and f0 != 0.0 and f1 != 0.0)
            converged = bool(abs(f0 - f1) <= 1e-6 * abs(f1))
            unreg = bool(np.isfinite(ge) and abs(gr - ge) <= 1e-7 * abs(ge))
            rows.append({"instance": q, "node": int(nd), "adjoint": float(gr), "fd": float(f0),
                         "rel": float(abs(gr - f0) / max(abs(f0), 1e-300)), "resolvable": resolvable,
                         "converged": converged, "unregularised": unreg,
                         "admissible": resolvable and converged and unreg})
    b.set_bathymetry(z0)
    summary("64 instances, 3.85M cells, 500 steps", rows)
    adm = [r for r in rows if r["admissible"]]
    assert len(adm) >= 8
    assert max(r["rel"] for r in adm) <= BOUND
