"""Batched discrete adjoint: a batch of instances of different sizes taped and
reversed together gives, instance by instance, the traces, dts and gradients
of the single-instance adjoint, and its initial-surface gradient matches
central finite differences of the forward run with the taped dts."""
import numpy as np
import pytest

from swe_fvm_gb300 import Fluxes, Solvers, SpaceDisc, TimeDisc, Wavespeeds, scenarios
from swe_fvm_gb300.adjoint import BatchRollout, Rollout

pytestmark = pytest.mark.gpu

N_STEPS, OBS, CKPT, CFL = 20, 4, 6, 0.3


def cases():
    out = []
    for q, (lat, seed) in enumerate([(25, 9), (18, 3), (30, 11)]):
        m, prim = scenarios.sloped_bump_case(lat, seed)
        g = np.random.default_rng(40 + q).choice(m.num_cells, 6, replace=False)
        out.append((m.contiguous(), prim, g))
    return out


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def runs():
    cs = cases()
    br = BatchRollout([c[0] for c in cs], [c[1] for c in cs], cfl=CFL)
    traces = br.forward(1, N_STEPS, CKPT, [c[2] for c in cs], OBS)
    dts = br.dts(N_STEPS)
    targets = [t * 0.97 + 0.002 for t in traces]
    grads = br.backward([2.0 * (t - tg) for t, tg in zip(traces, targets)])
    singles = []
    for q, (m, prim, g) in enumerate(cs):
        ro = Rollout(m, prim, cfl=CFL)
        tr = ro.forward(1, N_STEPS, CKPT, g, OBS)
        singles.append((tr, ro.dts(N_STEPS), ro.backward(2.0 * (tr - targets[q]))))
    return cs, traces, dts, targets, grads, singles


def test_batch_forward_equals_single(gpu, runs):
    cs, traces, dts, _, _, singles = runs
    for q in range(len(cs)):
        assert np.array_equal(traces[q], singles[q][0])
        assert np.array_equal(dts[:, q], singles[q][1])


def test_batch_gradients_equal_single(gpu, runs):
    cs, _, _, _, grads, singles = runs
    for q in range(len(cs)):
        gp, gz = grads[q]
        sp, sz = singles[q][2]
        assert rel(gp, sp) < 1e-12
        assert rel(gz, sz) < 1e-12


def test_batch_w0_gradient_finite_differences(gpu, runs):
    """Central differences (eps 1e-7) of each instance's loss through the plain
    GPU step with that instance's taped dts, at its wet cells with the largest
    gradient (the same criteria as the single-instance test)."""
    cs, _, dts, targets, grads, _ = runs
    eps = 1e-7
    errs = []
    for q, (m, prim, g) in enumerate(cs):
        gp = grads[q][0]
        wet = np.where(prim[:, 0] - m.centroids()[:, 2] > 0.02)[0]
        for c in wet[np.argsort(-np.abs(gp[wet, 0]))[:3]]:
            vals = []
            for sgn in (1.0, -1.0):
                p = prim.copy()
                p[c, 0] += sgn * eps
                sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p, cfl=CFL)
                td = TimeDisc(sd)
                tr = []
                for n in range(N_STEPS):
                    Solvers.SSPRK2(td, dts[n, q])
                    if (n + 1) % OBS == 0:
                        tr.append(sd.GetVolField()[g, 0])
                vals.append(float(np.sum((np.array(tr) - targets[q]) ** 2)))
            fd = (vals[0] - vals[1]) / (2 * eps)
            errs.append(abs(gp[c, 0] - fd) / max(abs(fd), 1e-30))
    # central differences at eps = 1e-7 of a bit-deterministic forward agree to
    # 1e-6 relative away from branch switches.  These instances have bumps
    # that emerge through the surface; two of the tested cells (measured:
    # 3.8e-5 and 2.9e-4) see partially-wet films in their domain of
    # dependence, where the reverse of PartWet1 is regularised below the depth
    # 1e-3 and branch switches lie within reach, so the bound on all cells is
    # looser than on the median
    assert np.median(errs) < 1e-6, errs
    assert max(errs) < 1e-3, errs
