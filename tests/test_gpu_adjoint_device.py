"""The autograd path keeps one device context per mesh and stays in device memory.

gauge_rollout / batch_gauge_rollout reuse the context they created on the
first call: a changed bed is written into it in place (swe_set_bathymetry),
the initial state is set from device memory, and traces and gradients are
device tensors.  Every call must give what a fresh context through the C ABI
gives (Rollout / BatchRollout): traces bit for bit and both gradients to
1e-12 of their largest entry (the bathymetry gradient's per-node sums use
atomics, so their order varies; a fresh and a reused context may also have
different device orders, which reorders a few other sums).
"""
import numpy as np
import pytest

from swe_fvm_gb300 import scenarios
from swe_fvm_gb300.adjoint import (BatchRollout, Rollout, batch_gauge_rollout, cache_info, clear_cache,
                                   gauge_rollout)
from swe_fvm_gb300.mesh import Mesh

pytestmark = pytest.mark.gpu

STEPS, OBS, CKPT = 200, 10, 50


def with_bed(m, z):
    g = m.geometry.copy()
    g[:, 2] = z
    return Mesh(g, m.edge_nodes, m.edge_cells, m.cell_nodes, m.cell_edges, m.cell_neighbours)


def close(a, b, tol=1e-12):
    return float(np.max(np.abs(a - b))) <= tol * max(float(np.max(np.abs(b))), 1e-300)


def test_gauge_rollout_reuses_one_context_on_the_adjoint_mesh(gpu):
    """Five forward/backward calls on the 250k-cell adjoint mesh with a
    different bed and initial surface each time: one context is created."""
    torch = pytest.importorskip("torch")
    mesh, prim = scenarios.hump_instance(2024, 250000)
    mesh = mesh.contiguous()
    gauges = np.random.default_rng(11).choice(mesh.num_cells, 64, replace=False)
    noise = np.random.default_rng(12).normal(size=mesh.num_nodes)
    z0 = mesh.geometry[:, 2].copy()
    bump = np.exp(-((mesh.centroids()[:, 0] - 0.5) ** 2) / 0.01)
    target = None
    clear_cache()
    n0 = cache_info()["created"]
    for k in range(5):
        zk = z0 * (1 + 0.01 * k * noise)
        pk = prim.copy()
        pk[:, 0] = np.maximum(prim[:, 0] + 0.001 * k * bump, with_bed(mesh, zk).centroids()[:, 2])
        ro = Rollout(with_bed(mesh, zk), pk)
        tr_ref = ro.forward(1, STEPS, CKPT, gauges, OBS)
        if target is None:
            target = tr_ref * 0.98 + 0.001
        gp, gz = ro.backward(2.0 * (tr_ref - target))
        del ro
        w0 = torch.tensor(pk[:, 0], device="cuda", requires_grad=True)
        z = torch.tensor(zk, device="cuda", requires_grad=True)
        tr = gauge_rollout(w0, z, mesh, gauges, STEPS, OBS, CKPT, uv0=pk[:, 1:])
        assert tr.is_cuda
        assert np.array_equal(tr.detach().cpu().numpy(), tr_ref), k
        loss = ((tr - torch.from_numpy(target).cuda()) ** 2).sum()
        loss.backward()
        assert w0.grad.is_cuda and z.grad.is_cuda
        assert close(w0.grad.cpu().numpy(), gp[:, 0]), k
        assert close(z.grad.cpu().numpy(), gz), k
    assert cache_info()["created"] - n0 == 1


def test_backward_after_another_forward_retapes(gpu):
    """Two forwards on the same context, then the first one's backward: the
    context re-tapes the first run before reversing it."""
    torch = pytest.importorskip("torch")
    m, prim = scenarios.sloped_bump_case(25, 9)
    m = m.contiguous()
    g = np.random.default_rng(5).choice(m.num_cells, 12, replace=False)
    clear_cache()
    n0 = cache_info()["created"]
    ro = Rollout(m, prim, cfl=0.3)
    tr_ref = ro.forward(1, 24, 10, g, 4)
    gp, _ = ro.backward(np.ones_like(tr_ref))
    w_a = torch.tensor(prim[:, 0], device="cuda", requires_grad=True)
    w_b = torch.tensor(prim[:, 0] + 1e-3, device="cuda", requires_grad=True)
    z = torch.tensor(m.geometry[:, 2], device="cuda")
    tr_a = gauge_rollout(w_a, z, m, g, 24, 4, 10, uv0=prim[:, 1:], cfl=0.3)
    tr_b = gauge_rollout(w_b, z, m, g, 24, 4, 10, uv0=prim[:, 1:], cfl=0.3)
    assert np.array_equal(tr_a.detach().cpu().numpy(), tr_ref)
    tr_a.sum().backward()
    assert close(w_a.grad.cpu().numpy(), gp[:, 0])
    assert cache_info()["created"] - n0 == 1
    del tr_b


def test_batch_gauge_rollout_matches_batch_rollout(gpu):
    torch = pytest.importorskip("torch")
    cases = [scenarios.sloped_bump_case(lat, seed) for lat, seed in [(25, 9), (18, 3), (30, 11)]]
    meshes = [c[0].contiguous() for c in cases]
    prims = [c[1] for c in cases]
    gauges = [np.random.default_rng(40 + q).choice(m.num_cells, 6, replace=False) for q, m in enumerate(meshes)]
    clear_cache()
    n0 = cache_info()["created"]
    for k in range(3):
        zs = [m.geometry[:, 2] * (1 + 0.002 * k) for m in meshes]
        br = BatchRollout([with_bed(m, z) for m, z in zip(meshes, zs)], prims, cfl=0.3)
        trs = br.forward(1, 20, 6, gauges, 4)
        grads = br.backward([np.ones_like(t) for t in trs])
        del br
        w0 = torch.tensor(np.concatenate([p[:, 0] for p in prims]), device="cuda", requires_grad=True)
        z = torch.tensor(np.concatenate(zs), device="cuda", requires_grad=True)
        tr = batch_gauge_rollout(w0, z, meshes, gauges, 20, 4, 6, uv0s=[p[:, 1:] for p in prims], cfl=0.3)
        assert np.array_equal(tr.detach().cpu().numpy(), np.concatenate(trs, axis=1)), k
        tr.sum().backward()
        assert close(w0.grad.cpu().numpy(), np.concatenate([gq[0][:, 0] for gq in grads])), k
        assert close(z.grad.cpu().numpy(), np.concatenate([gq[1] for gq in grads])), k
    assert cache_info()["created"] - n0 == 1


def test_set_bathymetry_equals_a_fresh_context(gpu):
    """A context whose bed was replaced steps exactly like one created with it."""
    from swe_fvm_gb300 import Fluxes, SpaceDisc, Wavespeeds

    m, prim = scenarios.random_front_case(30, seed=4)
    z1 = m.geometry[:, 2] * 0.9 + 0.01
    a = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    a.set_bathymetry(z1)
    a.prime()
    b = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), with_bed(m, z1), prim)
    assert a.GetMinLenToWavespeed() == b.GetMinLenToWavespeed()
    a.run_cfl(1, 20)
    b.run_cfl(1, 20)
    assert np.array_equal(a.GetVolField(), b.GetVolField())


def test_run_traces_repeats_the_taped_run(gpu):
    """The fixed-dt trace run with the dts a taped run recorded gives its traces."""
    m, prim = scenarios.sloped_bump_case(25, 9)
    g = np.random.default_rng(5).choice(m.num_cells, 12, replace=False)
    ro = Rollout(m, prim, cfl=0.3)
    tr = ro.forward(1, 24, 10, g, 4)
    dts = ro.dts(24)
    ro.sd.SetVolField(prim)
    assert np.array_equal(ro.sd.run_traces(1, dts, g, 4), tr)
