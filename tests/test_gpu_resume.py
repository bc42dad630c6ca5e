"""Checkpoint and resume: a run interrupted, saved (state, time and the CFL
ratio of its last flux pass), restored into a fresh context and continued
ends in the same state and time, bit for bit, as the uninterrupted run; batch
instances resume the same way."""
import numpy as np
import pytest

from swe_fvm_gb300 import Batch, Fluxes, SpaceDisc, Wavespeeds, scenarios

pytestmark = pytest.mark.gpu


def test_resumed_run_equals_the_uninterrupted_run(gpu, tmp_path):
    m, prim = scenarios.random_front_case(30, 5)
    a = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, cfl=0.3)
    ta = a.run_cfl(1, 20)
    b = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, cfl=0.3)
    b.run_cfl(1, 10)
    b.save(str(tmp_path / "ck.npz"), step=10)
    del b
    c = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, cfl=0.3)
    assert c.restore(str(tmp_path / "ck.npz")) == 10
    tc = c.run_cfl(1, 10)
    assert np.array_equal(c.GetVolField(), a.GetVolField())
    assert tc == ta == c.time()


def test_batch_instances_resume(gpu):
    """A batch created from checkpointed states, with their times set,
    continues exactly as the uninterrupted batch; set_prim stores a state
    bit for bit."""
    cases = [scenarios.random_front_case(14, 1), scenarios.random_front_case(18, 2)]
    fl = Fluxes.HLLC(Wavespeeds.Einfeldt)
    full = Batch([c[0] for c in cases], [c[1] for c in cases], fl, cfl=0.3)
    full.run_cfl(1, 12)
    half = Batch([c[0] for c in cases], [c[1] for c in cases], fl, cfl=0.3)
    half.run_cfl(1, 6)
    saved = [(half.prim(q), half.time(q), half.min_len_to_wavespeed(q)) for q in range(2)]
    resumed = Batch([c[0] for c in cases], [s[0] for s in saved], fl, cfl=0.3)
    for q, (p, t, r) in enumerate(saved):
        resumed.set_time(q, t)
        resumed.set_min_len_to_wavespeed(q, r)
    resumed.run_cfl(1, 6)
    for q in range(2):
        assert np.array_equal(resumed.prim(q), full.prim(q))
        assert resumed.time(q) == full.time(q)
    half.set_prim(1, full.prim(1))
    assert np.array_equal(half.prim(1), full.prim(1))
