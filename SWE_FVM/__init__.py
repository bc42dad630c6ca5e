"""The reference's Python module name (pybind/Topology.cpp:8-31 builds a module
``SWE_FVM`` exposing ``Topology``), over the GPU step.

``import SWE_FVM`` gives the reference's ``Topology`` (``Topology.create``
with the same six arguments, copying them instead of keeping references) and
the rest of the host API of ``swe_fvm_gb300``: ``Domain``, ``SpaceDisc``,
``TimeDisc``, ``Solvers``, ``Fluxes``, ``Wavespeeds``, the batched form and
the adjoint's ``gauge_rollout`` and ``batch_gauge_rollout`` (``torch.autograd.Function``s).
"""
from swe_fvm_gb300 import (  # noqa: F401
    SCHEMES,
    Batch,
    Domain,
    Fluxes,
    Solvers,
    SpaceDisc,
    SweError,
    TimeDisc,
    Topology,
    Wavespeeds,
)
from swe_fvm_gb300.adjoint import batch_gauge_rollout, gauge_rollout  # noqa: F401

__all__ = ["Topology", "Domain", "SpaceDisc", "TimeDisc", "Solvers", "Fluxes", "Wavespeeds", "Batch", "SweError",
           "SCHEMES", "gauge_rollout", "batch_gauge_rollout"]
