"""Discrete adjoint: gradients of a gauge-misfit loss with respect to the
initial surface level and the node bathymetry, checked by central finite
differences of the GPU forward run (dt frozen to the taped forward's) and of
the CPU restatement differenced the same way."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from swe_fvm_gb300 import Fluxes, Solvers, SpaceDisc, TimeDisc, Wavespeeds, scenarios
from swe_fvm_gb300.adjoint import Rollout
from swe_fvm_gb300.mesh import Mesh

pytestmark = pytest.mark.gpu

N_STEPS, OBS, CKPT = 24, 4, 10


def case():
    """A bed sloped everywhere with an emerging bump, a hump and a current
    (scenarios.sloped_bump_case): the finite differences are taken where no
    limiter, wet/dry or HLLC branch switch is within reach of the step."""
    m, prim = scenarios.sloped_bump_case(25, 9)
    rng = np.random.default_rng(5)
    gauges = rng.choice(m.num_cells, 12, replace=False)
    return m.contiguous(), prim, gauges


def loss_of(traces, target):
    return float(np.sum((traces - target) ** 2))


def gpu_traces(m, prim, dts, gauges):
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, cfl=0.3)
    td = TimeDisc(sd)
    out = []
    for n, dt in enumerate(dts):
        Solvers.SSPRK2(td, dt)
        if (n + 1) % OBS == 0:
            out.append(sd.GetVolField()[gauges, 0])
    return np.array(out)


def cpu_traces(m, prim, dts, gauges):
    o = Oracle(m, prim)
    out = []
    for n, dt in enumerate(dts):
        o.step("SSPRK2", dt)
        if (n + 1) % OBS == 0:
            out.append(o.prim()[gauges, 0])
    return np.array(out)


@pytest.fixture(scope="module")
def adjoint_run():
    m, prim, gauges = case()
    ro = Rollout(m, prim, cfl=0.3)
    traces = ro.forward(1, N_STEPS, CKPT, gauges, OBS)
    dts = ro.dts(N_STEPS)
    target = traces * 0.97 + 0.002
    gp, gz = ro.backward(2.0 * (traces - target))
    return m, prim, gauges, traces, target, dts, gp, gz


def test_taped_forward_equals_plain_steps(gpu, adjoint_run):
    m, prim, gauges, traces, target, dts, gp, gz = adjoint_run
    assert np.array_equal(traces, gpu_traces(m, prim, dts, gauges))
    assert np.array_equal(traces, cpu_traces(m, prim, dts, gauges))


def test_gradient_initial_surface_matches_central_differences(gpu, adjoint_run):
    m, prim, gauges, traces, target, dts, gp, gz = adjoint_run
    bc = m.centroids()[:, 2]
    wet = np.where(prim[:, 0] - bc > 0.02)[0]
    cand = wet[np.argsort(-np.abs(gp[wet, 0]))[:6]]
    eps = 1e-7
    errs = []
    for c in cand:
        fd = []
        for traces_fn in (gpu_traces, cpu_traces):
            p1 = prim.copy(); p1[c, 0] += eps
            p2 = prim.copy(); p2[c, 0] -= eps
            fd.append((loss_of(traces_fn(m, p1, dts, gauges), target) - loss_of(traces_fn(m, p2, dts, gauges), target)) / (2 * eps))
        assert fd[0] == fd[1]  # the CPU restatement differenced the same way
        errs.append(abs(gp[c, 0] - fd[0]) / max(abs(fd[0]), 1e-30))
    # central differences at eps = 1e-7 of a bit-deterministic forward: 1e-6
    # relative away from limiter, wet/dry and HLLC branch switches
    assert max(errs) < 1e-6, errs


def test_gradient_bathymetry_matches_central_differences(gpu, adjoint_run):
    """At nodes whose surrounding cells are all wet: at a node touching a dry
    cell (level exactly at the cell bathymetry) the loss has a kink, a one-sided
    perturbation turns the cell wet, and central differences are meaningless."""
    m, prim, gauges, traces, target, dts, gp, gz = adjoint_run
    h = prim[:, 0] - m.centroids()[:, 2]
    node_min_h = np.full(m.num_nodes, np.inf)
    np.minimum.at(node_min_h, m.cell_nodes.reshape(-1), np.repeat(h, 3))
    boundary = np.zeros(m.num_nodes, bool)
    boundary[m.edge_nodes[m.edge_cells[:, 1] < 0].reshape(-1)] = True
    ok = np.where((node_min_h > 0.02) & ~boundary)[0]
    cand = ok[np.argsort(-np.abs(gz[ok]))[:6]]
    eps = 1e-7
    errs = []
    for nd in cand:
        fd = []
        for sgn in (1, -1):
            g = m.geometry.copy()
            g[nd, 2] += sgn * eps
            mm = Mesh(g, m.edge_nodes, m.edge_cells, m.cell_nodes, m.cell_edges, m.cell_neighbours)
            fd.append(loss_of(gpu_traces(mm, prim, dts, gauges), target))
        d = (fd[0] - fd[1]) / (2 * eps)
        errs.append(abs(gz[nd] - d) / max(abs(d), 1e-30))
    # central differences at eps = 1e-7 of a bit-deterministic forward: 1e-6
    # relative away from limiter, wet/dry and HLLC branch switches
    assert max(errs) < 1e-6, errs


def test_autograd_function_matches_c_abi(gpu, adjoint_run):
    torch = pytest.importorskip("torch")
    from swe_fvm_gb300.adjoint import gauge_rollout

    m, prim, gauges, traces, target, dts, gp, gz = adjoint_run
    w0 = torch.tensor(prim[:, 0], dtype=torch.float64, device="cuda", requires_grad=True)
    z = torch.tensor(m.geometry[:, 2], dtype=torch.float64, device="cuda", requires_grad=True)
    tr = gauge_rollout(w0, z, m, gauges, N_STEPS, OBS, CKPT, uv0=prim[:, 1:], cfl=0.3)
    assert np.array_equal(tr.detach().cpu().numpy(), traces)
    loss = ((tr - torch.from_numpy(target).cuda()) ** 2).sum()
    loss.backward()
    assert np.allclose(w0.grad.cpu().numpy(), gp[:, 0], rtol=1e-12, atol=1e-300)
    # the bathymetry gradient sums with atomics: equal up to the summation order
    assert np.linalg.norm(z.grad.cpu().numpy() - gz) <= 1e-12 * np.linalg.norm(gz)


@pytest.mark.parametrize("flux", [0, 1])
@pytest.mark.parametrize("ws", [0, 1, 2])
def test_hand_flux_reverse_equals_dual_jacobian(gpu, flux, ws):
    import ctypes

    from swe_fvm_gb300 import _lib

    err = ctypes.c_double(-1.0)
    assert _lib.load().swe_selftest_flux_adjoint(flux, ws, 1 << 20, 7, ctypes.byref(err)) == 0
    assert err.value < 1e-9, err.value
