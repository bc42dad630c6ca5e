"""ctypes wrapper around the C restatement in swe_oracle.c.

TEST INFRASTRUCTURE ONLY: the checker for the GPU library and the timed CPU
baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "swe_oracle.c")

JACOBI, LITERAL = 0, 1
FLUX = {"HLL": 0, "HLLC": 1}
WAVESPEED = {"Rusanov": 0, "Davis": 1, "Einfeldt": 2}
SCHEME = {"Euler": 0, "SSPRK2": 1, "SSPRK3": 2}


def build(force: bool = False) -> str:
    """Compile the restatement with gcc: -O3, no FMA contraction, no -march,
    OpenMP for the optional jacobi-order threads."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
                           "-shared", SRC, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        d, i64, i32, vp = ctypes.c_double, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [i64, i64, i64, vp, vp, vp, vp, vp, vp, vp, i32, i32, d, d, i32]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_step.argtypes = [vp, i32, d]
        L.oracle_step_table.argtypes = [vp, i32, vp, vp, vp, d]
        L.oracle_compute_interface_values.argtypes = [vp]
        L.oracle_compute_fluxes.argtypes = [vp]
        L.oracle_min_len_to_wavespeed.argtypes = [vp]
        L.oracle_min_len_to_wavespeed.restype = d
        L.oracle_set_threads.argtypes = [vp, i32]
        L.oracle_get_prim.argtypes = [vp, vp]
        L.oracle_set_prim.argtypes = [vp, vp]
        L.oracle_get_edge_fields.argtypes = [vp, vp, vp, vp, vp]
        L.oracle_classify.argtypes = [vp, vp]
        L.oracle_wavespeed.argtypes = [i32, d, d, d, d, vp]
        L.oracle_bisection_cubic.argtypes = [d, d, d, d, d]
        L.oracle_bisection_cubic.restype = d
        L.oracle_gradient3.argtypes = [vp, vp, vp, vp]
        L.oracle_prim_assign.argtypes = [d, vp, vp]
        L.oracle_cons_assign.argtypes = [d, vp, vp]
        L.oracle_cbrt_rn.argtypes = [d]
        L.oracle_cbrt_rn.restype = d
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """One SpaceDisc + TimeDisc pair of the restated reference solver."""

    def __init__(self, mesh, prim0, flux="HLLC", wavespeed="Einfeldt", cor=0.0, tau=0.0, order=JACOBI):
        L = lib()
        m = mesh.contiguous()
        self._keep = m
        self.mesh = m
        p0 = np.ascontiguousarray(prim0, dtype=np.float64)
        self.ptr = L.oracle_create(m.num_nodes, m.num_edges, m.num_cells, _p(m.geometry), _p(m.edge_nodes),
                                   _p(m.edge_cells), _p(m.cell_nodes), _p(m.cell_edges), _p(m.cell_neighbours),
                                   _p(p0), FLUX[flux], WAVESPEED[wavespeed], float(cor), float(tau), int(order))

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().oracle_destroy(self.ptr)
            self.ptr = None

    def step(self, scheme="SSPRK2", dt=1e-3):
        lib().oracle_step(self.ptr, SCHEME[scheme], float(dt))

    def step_table(self, a, b, c, dt):
        """One step of a Shu-Osher table (stage s: a[s] U0 + b[s] U_{s-1} +
        RHS(U_{s-1}, c[s] dt))."""
        a, b, c = (np.ascontiguousarray(x, dtype=np.float64) for x in (a, b, c))
        lib().oracle_step_table(self.ptr, len(a), _p(a), _p(b), _p(c), float(dt))

    def compute_interface_values(self):
        lib().oracle_compute_interface_values(self.ptr)

    def compute_fluxes(self):
        lib().oracle_compute_fluxes(self.ptr)

    def min_len_to_wavespeed(self) -> float:
        return lib().oracle_min_len_to_wavespeed(self.ptr)

    def set_threads(self, n: int) -> None:
        """Run the jacobi-order loops on n OpenMP threads (results unchanged)."""
        lib().oracle_set_threads(self.ptr, int(n))

    def prim(self) -> np.ndarray:
        out = np.empty((self.mesh.num_cells, 3))
        lib().oracle_get_prim(self.ptr, _p(out))
        return out

    def set_prim(self, prim):
        a = np.ascontiguousarray(prim, dtype=np.float64)
        lib().oracle_set_prim(self.ptr, _p(a))

    def edge_fields(self):
        E, N = self.mesh.num_edges, self.mesh.num_nodes
        edg = np.empty((2 * E, 3))
        src = np.empty((2 * E, 3))
        f = np.empty((E, 3))
        mx = np.empty(N)
        lib().oracle_get_edge_fields(self.ptr, _p(edg), _p(src), _p(f), _p(mx))
        return edg, src, f, mx

    def classify(self) -> np.ndarray:
        out = np.empty(self.mesh.num_cells, dtype=np.int32)
        lib().oracle_classify(self.ptr, _p(out))
        return out
