"""Device orders and block sizes change nothing but speed: on a mesh whose
cells, edges and nodes are numbered at random, every reorder strategy and
every block size gives the same state bit for bit (and the oracle's), the
debug getters and the adjoint answer in the caller's numbering, and the tuner
reports what it chose."""
import numpy as np
import pytest

from helpers import shuffle_mesh
from oracle.oracle import JACOBI, Oracle
from swe_fvm_gb300 import Batch, Fluxes, SpaceDisc, Wavespeeds, scenarios
from swe_fvm_gb300.adjoint import BatchRollout, Rollout

pytestmark = pytest.mark.gpu

STRATEGIES = ["keep", "morton", "rcm", "auto"]


@pytest.fixture(scope="module")
def case():
    m, prim = scenarios.random_front_case(40, 3)
    m = m.contiguous()
    s, pc, pe, pn = shuffle_mesh(m, 5)
    return m, prim, s, prim[pc], pc, pe, pn


def _run(mesh, prim, n, reorder="auto", block=0, scheme=1):
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), mesh, prim, cfl=0.3, reorder=reorder, block=block)
    t = sd.run_cfl(scheme, n)
    return sd, t


def test_every_order_gives_the_same_state(gpu, case):
    m, prim, s, sprim, pc, pe, pn = case
    ref, t_ref = _run(m, prim, 25, reorder="keep")
    want = ref.GetVolField()[pc]
    ints = None
    for strategy in STRATEGIES:
        sd, t = _run(s, sprim, 25, reorder=strategy)
        assert np.array_equal(sd.GetVolField(), want), strategy
        assert t == t_ref, strategy
        # the integrals visit cells in the caller's order in every layout
        ints = sd.integrals() if ints is None else ints
        assert np.array_equal(sd.integrals(), ints), strategy
    assert _run(s, sprim, 1, reorder="auto")[0].tuning()["reorder"] in ("morton", "rcm")


def test_reordered_run_matches_the_oracle(gpu, case):
    m, prim, s, sprim, pc, pe, pn = case
    o = Oracle(s, sprim, flux="HLLC", wavespeed="Einfeldt", order=JACOBI)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), s, sprim, reorder="morton")
    o.compute_interface_values()
    o.compute_fluxes()
    for _ in range(5):
        dt = 0.15 * o.min_len_to_wavespeed()
        o.step("SSPRK2", dt)
        sd.run(1, dt, 1)
        assert np.array_equal(sd.GetVolField(), o.prim())


def test_getters_answer_in_the_callers_numbering(gpu, case):
    m, prim, s, sprim, pc, pe, pn = case
    for strategy in ("morton", "rcm"):
        a = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), s, sprim, reorder="keep")
        b = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), s, sprim, reorder=strategy)
        for sd in (a, b):
            sd.run(1, 1e-3, 3)
            sd.ComputeInterfaceValues()
            sd.ComputeFluxes()
        assert np.array_equal(a.GetEdgField(), b.GetEdgField()), strategy
        assert np.array_equal(a.GetSrcField(), b.GetSrcField()), strategy
        assert np.array_equal(a.GetFluxes(), b.GetFluxes()), strategy
        assert np.array_equal(a.GetNodeMax(), b.GetNodeMax()), strategy
        assert a.GetMinLenToWavespeed() == b.GetMinLenToWavespeed()


def test_device_state_io_in_the_callers_order(gpu, case):
    import torch

    m, prim, s, sprim, pc, pe, pn = case
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), s, sprim, reorder="morton")
    x = torch.empty((s.num_cells, 3), dtype=torch.float64, device="cuda")
    sd.get_prim_device(x.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(x.cpu().numpy(), sprim)
    y = torch.from_numpy(sprim[::-1].copy()).cuda()
    sd.set_prim_device(y.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(sd.GetVolField(), sprim[::-1])


@pytest.mark.parametrize("block", [32, 64, 128, 256])
def test_block_sizes_give_the_same_state(gpu, case, block):
    m, prim, s, sprim, pc, pe, pn = case
    ref = _run(s, sprim, 12, reorder="keep", block=256)[0].GetVolField()
    sd, _ = _run(s, sprim, 12, reorder="keep", block=block)
    assert np.array_equal(sd.GetVolField(), ref)
    tu = sd.tuning()
    assert (tu["block_recon"], tu["block_flux"], tu["block_update"]) == (block, block, block)


def test_tuned_blocks_are_reported(gpu):
    m, prim = scenarios.dam_break(120)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    tu = sd.tuning()
    assert {tu["block_recon"], tu["block_flux"], tu["block_update"]} <= {64, 128, 256}
    # tuning ran on a copy: the state and the CFL ratio are the initial ones
    assert np.array_equal(sd.GetVolField(), prim)
    fixed = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, block=256)
    assert sd.GetMinLenToWavespeed() == fixed.GetMinLenToWavespeed()
    sd.run_cfl(1, 10)
    fixed.run_cfl(1, 10)
    assert np.array_equal(sd.GetVolField(), fixed.GetVolField())


def test_batch_instances_keep_their_own_order(gpu, case):
    m, prim, s, sprim, pc, pe, pn = case
    cases = [(s, sprim), (m, prim), (s, sprim)]
    b = Batch([c[0] for c in cases], [c[1] for c in cases], Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.3)
    b.run_cfl(1, 10)
    for q, (mq, pq) in enumerate(cases):
        sd, t = _run(mq, pq, 10, reorder="keep")
        assert np.array_equal(b.prim(q), sd.GetVolField()), q
        assert b.time(q) == t


def test_adjoint_in_the_callers_numbering(gpu, case):
    m, prim, s, sprim, pc, pe, pn = case
    rng = np.random.default_rng(2)
    gauges = rng.choice(s.num_cells, 6, replace=False)
    out = {}
    for strategy in ("keep", "morton"):
        r = Rollout(s, sprim, cfl=0.3, reorder=strategy)
        tr = r.forward(1, 40, 10, gauges, 5)
        gp, gz = r.backward(np.ones_like(tr))
        out[strategy] = (tr, r.dts(40), gp, gz)
    (ta, da, ga, za), (tb, db, gb, zb) = out["keep"], out["morton"]
    assert np.array_equal(ta, tb)
    assert np.array_equal(da, db)
    # sums over cells run in another order: equal to round-off
    assert np.max(np.abs(ga - gb)) <= 1e-12 * max(1.0, np.max(np.abs(ga)))
    assert np.max(np.abs(za - zb)) <= 1e-12 * max(1.0, np.max(np.abs(za)))
    assert np.max(np.abs(ga)) > 0


def test_batch_adjoint_gauges_in_the_callers_numbering(gpu, case):
    m, prim, s, sprim, pc, pe, pn = case
    g = [np.array([3, 50, 400]), np.array([7, 9])]
    outs = []
    for strategy in ("keep", "auto"):
        br = BatchRollout([s, m], [sprim, prim], cfl=0.3, reorder=strategy)
        tr = br.forward(1, 20, 5, g, 4)
        outs.append((tr, br.backward([np.ones_like(t) for t in tr])))
    for q in range(2):
        assert np.array_equal(outs[0][0][q], outs[1][0][q])
        for a, b in zip(outs[0][1][q], outs[1][1][q]):
            assert np.max(np.abs(a - b)) <= 1e-12 * max(1.0, np.max(np.abs(a)))


def test_timed_order_choice_on_a_large_mesh(gpu):
    """From 65,536 cells up, AUTO times the three orders; whichever it keeps,
    the state is the caller-order state."""
    m, prim = scenarios.dam_break(190)
    assert m.num_cells >= 1 << 16
    s, pc, _, _ = shuffle_mesh(m.contiguous(), 9)
    a, ta = _run(s, prim[pc], 6, reorder="auto")
    k, tk = _run(s, prim[pc], 6, reorder="keep")
    assert a.tuning()["reorder"] in ("keep", "morton", "rcm")
    assert np.array_equal(a.GetVolField(), k.GetVolField())
    assert ta == tk
    assert np.array_equal(a.integrals(), k.integrals())


def test_timed_order_choice_for_a_large_batch(gpu):
    """A batch of 65,536 cells or more times one order for all instances; each
    instance still equals its single context."""
    cases = [scenarios.dam_break(120, seed_mesh=q) for q in range(3)]
    assert sum(c[0].num_cells for c in cases) >= 1 << 16
    b = Batch([c[0] for c in cases], [c[1] for c in cases], Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.3)
    orders = {b.tuning(q)["reorder"] for q in range(3)}
    assert len(orders) == 1 and orders <= {"keep", "morton", "rcm"}
    b.run_cfl(1, 8)
    for q, (m, p) in enumerate(cases):
        sd, t = _run(m, p, 8, reorder="keep")
        assert np.array_equal(b.prim(q), sd.GetVolField()), q
        assert b.time(q) == t
