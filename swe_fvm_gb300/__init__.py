"""GB300-native explicit finite-volume shallow-water step (FP64).

The compute path is libswe_gb300.so: hand-written sm_103a kernels behind the
C ABI of include/swe_fvm_gb300.h.  This package is the host side: a ctypes
binding, a mirror of the reference's SpaceDisc / TimeDisc / Solvers / Fluxes
API, mesh and workload generators, and the PyTorch autograd layer.
"""
from .mesh import Mesh, build_topology, structured_square, jittered_delaunay  # noqa: F401
from .solver import (  # noqa: F401
    REORDER,
    SCHEMES,
    Batch,
    Domain,
    Fluxer,
    Fluxes,
    Solvers,
    SpaceDisc,
    SweError,
    TimeDisc,
    Topology,
    Wavespeeds,
    layout_plan,
    ssprk_m2,
)

__version__ = "0.1.0"
