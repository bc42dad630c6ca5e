"""Runs a fixed set of steps and prints one JSON line of state digests; run
once with the product library and once with SWE_GB300_CHECKED=1 (the build
whose step kernels range-check every gathered index) by test_gpu_checked."""
import hashlib
import json
import sys

import numpy as np

from swe_fvm_gb300 import Batch, Fluxes, SpaceDisc, Wavespeeds, _lib, scenarios
from swe_fvm_gb300.mesh import shuffled


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    out = {"checked": _lib.checked(), "library": _lib.library_path()}
    cases = {"front": scenarios.random_front_case(30, 3), "bump": scenarios.sloped_bump_case(20, 4),
             "dam": scenarios.dam_break(40)}
    for name, (m, prim) in cases.items():
        for flux in (Fluxes.HLLC(Wavespeeds.Einfeldt), Fluxes.HLL(Wavespeeds.Rusanov)):
            for scheme in (0, 1, 2):
                sd = SpaceDisc(flux, m, prim, cfl=0.3)
                t = sd.run_cfl(scheme, 15)
                sd.synchronize()  # raises on any device error bit
                out[f"{name}/{flux.kind}{flux.wavespeed}/{scheme}"] = [digest(sd.GetVolField()), t]
    m, prim = cases["front"]
    s, cf, _, _ = shuffled(m.contiguous(), 2)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), s, prim[cf], cfl=0.3, reorder="rcm")
    sd.run_cfl(1, 15)
    sd.synchronize()
    out["shuffled/rcm"] = digest(sd.GetVolField())
    b = Batch([c[0] for c in cases.values()], [c[1] for c in cases.values()], Fluxes.HLLC(Wavespeeds.Einfeldt),
              cfl=0.3)
    b.run_cfl(1, 15)
    b.synchronize()
    out["batch"] = [digest(b.prim(q)) for q in range(len(cases))]
    # the discrete adjoint: traces exactly, gradients through sums whose
    # atomic order may differ between runs (compared to round-off by the test)
    from swe_fvm_gb300.adjoint import Rollout

    m, prim = cases["bump"]
    gauges = np.random.default_rng(4).choice(m.num_cells, 8, replace=False)
    ro = Rollout(m, prim, cfl=0.3)
    tr = ro.forward(1, 20, 8, gauges, 4)
    gp, gz = ro.backward(np.ones_like(tr))
    ro.sd.synchronize()
    out["adjoint_traces"] = digest(tr)
    out["adjoint_grads"] = [float(np.abs(gp).sum()), float(np.abs(gz).sum()), float(np.abs(gp).max()),
                            float(np.abs(gz).max())]
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
