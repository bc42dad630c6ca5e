"""ctypes wrapper around oracle/_ref/libswe_ref.so: the reference's own solver.

TEST INFRASTRUCTURE ONLY.  The library is the reference's src/*.cpp compiled
here by oracle/ref/build_ref.py (against oracle/eigen_subset, Q1 and Q20
patched) with the driver oracle/ref/ref_driver.cpp.  It can only be built
where the reference sources are present; tests that need it skip elsewhere,
and the GPU tests use the golden vectors it wrote into tests/golden instead.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from oracle.ref import build_ref

JACOBI, LITERAL = 0, 1
FLUX = {"HLL": 0, "HLLC": 1}
WAVESPEED = {"Rusanov": 0, "Davis": 1, "Einfeldt": 2}
SCHEME = {"Euler": 0, "SSPRK2": 1, "SSPRK3": 2}

_libs = {}


def available() -> bool:
    return build_ref.available() or os.path.exists(build_ref.LIB)


def lib(q20_literal: bool = False):
    """The reference build; q20_literal selects the build whose positivity
    test (src/MUSCLObject.cpp:68) is left as Eigen's release build reads it."""
    key = bool(q20_literal)
    if key not in _libs:
        if build_ref.available():
            build_ref.build()
        path = build_ref.LIB_Q20LIT if key else build_ref.LIB
        L = ctypes.CDLL(path)
        d, i64, i32, vp = ctypes.c_double, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
        L.swe_ref_create.restype = vp
        L.swe_ref_create.argtypes = [i64, i64, i64, vp, vp, vp, vp, vp, vp, vp, i32, i32, d, i32]
        L.swe_ref_destroy.argtypes = [vp]
        L.swe_ref_step.argtypes = [vp, i32, d]
        L.swe_ref_step.restype = i32
        L.swe_ref_interface.argtypes = [vp]
        L.swe_ref_interface.restype = i32
        L.swe_ref_error.argtypes = [vp]
        L.swe_ref_error.restype = ctypes.c_char_p
        L.swe_ref_min_len_to_wavespeed.argtypes = [vp]
        L.swe_ref_min_len_to_wavespeed.restype = d
        L.swe_ref_cfl_dt.argtypes = [vp]
        L.swe_ref_cfl_dt.restype = d
        L.swe_ref_get_prim.argtypes = [vp, vp]
        L.swe_ref_set_prim.argtypes = [vp, vp]
        L.swe_ref_get_edge_fields.argtypes = [vp, vp, vp, vp, vp]
        L.swe_ref_classify.argtypes = [vp, vp]
        _libs[key] = L
    return _libs[key]


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Reference:
    """One SpaceDisc + TimeDisc pair of the reference solver itself."""

    def __init__(self, mesh, prim0, flux="HLLC", wavespeed="Einfeldt", cor=0.0, order=JACOBI, q20_literal=False):
        self._L = lib(q20_literal)
        m = mesh.contiguous()
        self.mesh = m
        p0 = np.ascontiguousarray(prim0, dtype=np.float64)
        self.ptr = self._L.swe_ref_create(m.num_nodes, m.num_edges, m.num_cells, _p(m.geometry), _p(m.edge_nodes),
                                          _p(m.edge_cells), _p(m.cell_nodes), _p(m.cell_edges),
                                          _p(m.cell_neighbours), _p(p0), FLUX[flux], WAVESPEED[wavespeed],
                                          float(cor), int(order))
        if not self.ptr:
            raise RuntimeError("the reference solver could not be constructed")

    def __del__(self):
        if getattr(self, "ptr", None):
            self._L.swe_ref_destroy(self.ptr)
            self.ptr = None

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self._L.swe_ref_error(self.ptr).decode())

    def step(self, scheme="SSPRK2", dt=1e-3):
        self._check(self._L.swe_ref_step(self.ptr, SCHEME[scheme], float(dt)))

    def interface(self):
        """SpaceDisc::ComputeInterfaceValues + ComputeFluxes."""
        self._check(self._L.swe_ref_interface(self.ptr))

    def min_len_to_wavespeed(self) -> float:
        return self._L.swe_ref_min_len_to_wavespeed(self.ptr)

    def cfl_dt(self) -> float:
        return self._L.swe_ref_cfl_dt(self.ptr)

    def prim(self) -> np.ndarray:
        out = np.empty((self.mesh.num_cells, 3))
        self._L.swe_ref_get_prim(self.ptr, _p(out))
        return out

    def set_prim(self, prim):
        a = np.ascontiguousarray(prim, dtype=np.float64)
        self._L.swe_ref_set_prim(self.ptr, _p(a))

    def edge_fields(self):
        E, N = self.mesh.num_edges, self.mesh.num_nodes
        edg = np.empty((2 * E, 3))
        src = np.empty((2 * E, 3))
        f = np.empty((E, 3))
        mx = np.empty(N)
        self._L.swe_ref_get_edge_fields(self.ptr, _p(edg), _p(src), _p(f), _p(mx))
        return edg, src, f, mx

    def classify(self) -> np.ndarray:
        out = np.empty(self.mesh.num_cells, dtype=np.int32)
        self._L.swe_ref_classify(self.ptr, _p(out))
        return out
