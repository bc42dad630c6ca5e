"""Streams: a context or batch moved to a caller's stream (PyTorch's here)
right after creation, or between runs, orders its earlier work before the
later work and gives the same state as on its own stream."""
import numpy as np
import pytest

from swe_fvm_gb300 import Batch, Fluxes, SpaceDisc, Wavespeeds, scenarios

pytestmark = pytest.mark.gpu


def test_moving_to_a_caller_stream_keeps_the_results(gpu):
    import torch

    m, prim = scenarios.dam_break(200)  # 79k cells: the timed device-order choice runs at creation
    ref = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    t_ref = ref.run_cfl(1, 10)
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim)
    sd.set_stream(s1.cuda_stream)  # straight after creation
    sd.run_cfl(1, 4)
    sd.set_stream(s2.cuda_stream)  # between runs, with s1 work possibly in flight
    sd.run_cfl(1, 3)
    sd.set_stream(0)               # back to the context's own stream
    t = sd.run_cfl(1, 3)
    assert np.array_equal(sd.GetVolField(), ref.GetVolField())
    assert t == t_ref


def test_batch_on_a_caller_stream(gpu):
    import torch

    cases = [scenarios.random_front_case(20, q) for q in range(3)]
    a = Batch([c[0] for c in cases], [c[1] for c in cases], Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.3)
    a.run_cfl(1, 8)
    s = torch.cuda.Stream()
    b = Batch([c[0] for c in cases], [c[1] for c in cases], Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.3)
    b.set_stream(s.cuda_stream)
    b.run_cfl(1, 8)
    s.synchronize()
    for q in range(3):
        assert np.array_equal(a.prim(q), b.prim(q))


def test_distinct_contexts_run_concurrently_from_host_threads(gpu):
    """One context per host thread (each on its own stream): creation, tuning,
    graph capture and runs proceed side by side and give the sequential
    results."""
    import threading

    cases = [scenarios.random_front_case(24, q) for q in range(4)] + [scenarios.dam_break(190)]
    want = []
    for m, p in cases:
        sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p, cfl=0.3)
        want.append((sd.run_cfl(1, 12), sd.GetVolField()))
    got = [None] * len(cases)
    errors = []

    def work(q):
        try:
            m, p = cases[q]
            sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p, cfl=0.3)
            got[q] = (sd.run_cfl(1, 12), sd.GetVolField())
        except Exception as ex:  # reported below
            errors.append(repr(ex))

    threads = [threading.Thread(target=work, args=(q,)) for q in range(len(cases))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    assert not errors, errors
    for q in range(len(cases)):
        assert got[q][0] == want[q][0]
        assert np.array_equal(got[q][1], want[q][1]), q
