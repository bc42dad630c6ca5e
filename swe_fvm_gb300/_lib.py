"""ctypes binding of libswe_gb300.so (the C ABI in include/swe_fvm_gb300.h).

There is no fallback: if the library cannot be built or loaded, every entry
point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_lib = None

SWE_OK = 0
STATUS_NAMES = {
    0: "SWE_OK",
    1: "SWE_ERR_INVALID_ARGUMENT",
    2: "SWE_ERR_INVALID_MESH",
    3: "SWE_ERR_NONFINITE",
    4: "SWE_ERR_TIMEOUT",
    5: "SWE_ERR_CUDA",
    6: "SWE_ERR_OUT_OF_MEMORY",
    7: "SWE_ERR_UNSUPPORTED",
}

# every symbol declared in include/swe_fvm_gb300.h
EXPORTS = [
    "swe_params_default", "swe_create", "swe_destroy", "swe_set_stream", "swe_step", "swe_run", "swe_run_cfl",
    "swe_cfl_dt", "swe_min_len_to_wavespeed", "swe_compute_interface_values", "swe_compute_fluxes",
    "swe_get_prim", "swe_set_prim", "swe_get_prim_device", "swe_set_prim_device", "swe_get_edge_values",
    "swe_get_fluxes", "swe_get_node_max", "swe_time_kernels", "swe_measure_fp64_peak", "swe_selftest_fp64", "swe_selftest_flux_adjoint", "swe_num_cells", "swe_launch_count", "swe_synchronize",
    "swe_last_error", "swe_adjoint_forward", "swe_adjoint_backward", "swe_adjoint_dts", "swe_edge_fluxes_noalloc", "swe_batch_create", "swe_batch_destroy", "swe_batch_set_stream", "swe_batch_run_cfl", "swe_batch_run",
    "swe_batch_get_prim", "swe_batch_time", "swe_batch_launch_count", "swe_batch_synchronize",
    "swe_batch_last_error", "swe_batch_adjoint_forward", "swe_batch_adjoint_backward", "swe_batch_adjoint_dts",
    "swe_integrals", "swe_batch_integrals", "swe_get_tuning", "swe_batch_get_tuning", "swe_layout_plan",
    "swe_set_scheme", "swe_batch_set_scheme", "swe_get_time", "swe_set_time", "swe_batch_set_time",
    "swe_batch_set_prim", "swe_set_min_len_to_wavespeed", "swe_batch_min_len_to_wavespeed",
    "swe_batch_set_min_len_to_wavespeed", "swe_adjoint_forward_device", "swe_adjoint_backward_device",
    "swe_run_traces", "swe_set_bathymetry", "swe_prime", "swe_batch_adjoint_forward_device",
    "swe_batch_adjoint_backward_device", "swe_batch_run_traces", "swe_batch_set_bathymetry", "swe_batch_prime",
    "swe_batch_set_prim_device", "swe_adjoint_set_regularisation", "swe_batch_adjoint_set_regularisation",
    "swe_adjoint_prepare", "swe_batch_adjoint_prepare",
]


class SweMesh(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int64),
        ("num_edges", ctypes.c_int64),
        ("num_cells", ctypes.c_int64),
        ("geometry", ctypes.c_void_p),
        ("edge_nodes", ctypes.c_void_p),
        ("edge_cells", ctypes.c_void_p),
        ("cell_nodes", ctypes.c_void_p),
        ("cell_edges", ctypes.c_void_p),
        ("cell_neighbours", ctypes.c_void_p),
    ]


class SweParams(ctypes.Structure):
    _fields_ = [
        ("flux", ctypes.c_int32),
        ("wavespeed", ctypes.c_int32),
        ("cor", ctypes.c_double),
        ("tau", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("reorder", ctypes.c_int32),
        ("block", ctypes.c_int32),
    ]


class SweError(RuntimeError):
    """A non-OK status from the C ABI."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


def checked() -> bool:
    """SWE_GB300_CHECKED=1 selects the checked build (device range checks on
    every gathered index of the step kernels) for this process."""
    return os.environ.get("SWE_GB300_CHECKED", "0") == "1"


def library_path() -> str:
    return _build.LIB_CHECKED if checked() else _build.LIB


def load(build_if_needed: bool = True):
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if build_if_needed:
        _build.build(checked=checked())
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with swe_fvm_gb300.build.build()")
    L = ctypes.CDLL(path)
    vp, d, i32, i64 = ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_int64
    P = ctypes.POINTER
    sig = {
        "swe_params_default": [P(SweParams)],
        "swe_create": [P(SweMesh), vp, P(SweParams), P(vp)],
        "swe_destroy": [vp],
        "swe_set_stream": [vp, vp],
        "swe_step": [vp, i32, d],
        "swe_run": [vp, i32, d, i64],
        "swe_run_cfl": [vp, i32, i64, vp],
        "swe_cfl_dt": [vp, P(d)],
        "swe_min_len_to_wavespeed": [vp, P(d)],
        "swe_compute_interface_values": [vp],
        "swe_compute_fluxes": [vp],
        "swe_get_prim": [vp, vp],
        "swe_set_prim": [vp, vp],
        "swe_get_prim_device": [vp, vp],
        "swe_set_prim_device": [vp, vp],
        "swe_get_edge_values": [vp, vp, vp],
        "swe_get_fluxes": [vp, vp],
        "swe_get_node_max": [vp, vp],
        "swe_time_kernels": [vp, i32, i64, vp],
        "swe_measure_fp64_peak": [P(d)],
        "swe_selftest_fp64": [i64, ctypes.c_uint64, P(i64), P(i64)],
        "swe_selftest_flux_adjoint": [i32, i32, i64, ctypes.c_uint64, P(d)],
        "swe_num_cells": [vp, P(i64)],
        "swe_launch_count": [vp, P(i64)],
        "swe_synchronize": [vp],
        "swe_last_error": [vp],
        "swe_edge_fluxes_noalloc": [i32, i32, i64, vp, vp, vp, d, vp, vp, vp],
        "swe_adjoint_forward": [vp, i32, i64, i64, i32, vp, i64, vp],
        "swe_adjoint_backward": [vp, vp, vp, vp],
        "swe_adjoint_dts": [vp, vp],
        "swe_batch_create": [i32, vp, vp, P(SweParams), i32, P(vp)],
        "swe_batch_destroy": [vp],
        "swe_batch_set_stream": [vp, vp],
        "swe_batch_run_cfl": [vp, i32, i64],
        "swe_batch_run": [vp, i32, d, i64],
        "swe_batch_get_prim": [vp, i32, vp],
        "swe_batch_time": [vp, i32, P(d)],
        "swe_batch_launch_count": [vp, P(i64)],
        "swe_batch_synchronize": [vp],
        "swe_batch_last_error": [vp],
        "swe_batch_adjoint_forward": [vp, i32, i64, i64, i32, vp, i64, vp],
        "swe_batch_adjoint_backward": [vp, vp, vp, vp],
        "swe_batch_adjoint_dts": [vp, vp],
        "swe_integrals": [vp, vp],
        "swe_batch_integrals": [vp, i32, vp],
        "swe_get_tuning": [vp, vp],
        "swe_batch_get_tuning": [vp, i32, vp],
        "swe_layout_plan": [vp, i32, vp, vp, vp, vp, P(i32)],
        "swe_set_scheme": [vp, i32, vp, vp, vp],
        "swe_batch_set_scheme": [vp, i32, vp, vp, vp],
        "swe_get_time": [vp, P(d)],
        "swe_set_time": [vp, d],
        "swe_batch_set_time": [vp, i32, d],
        "swe_batch_set_prim": [vp, i32, vp],
        "swe_set_min_len_to_wavespeed": [vp, d],
        "swe_batch_min_len_to_wavespeed": [vp, i32, P(d)],
        "swe_batch_set_min_len_to_wavespeed": [vp, i32, d],
        "swe_adjoint_forward_device": [vp, i32, i64, i64, i32, vp, i64, vp],
        "swe_adjoint_backward_device": [vp, vp, vp, vp],
        "swe_run_traces": [vp, i32, i64, vp, i32, vp, i64, vp],
        "swe_set_bathymetry": [vp, vp],
        "swe_prime": [vp],
        "swe_batch_adjoint_forward_device": [vp, i32, i64, i64, i32, vp, i64, vp],
        "swe_batch_adjoint_backward_device": [vp, vp, vp, vp],
        "swe_batch_run_traces": [vp, i32, i64, vp, i32, vp, i64, vp],
        "swe_batch_set_bathymetry": [vp, vp],
        "swe_batch_prime": [vp],
        "swe_batch_set_prim_device": [vp, i32, vp],
        "swe_adjoint_set_regularisation": [vp, d],
        "swe_batch_adjoint_set_regularisation": [vp, d],
        "swe_adjoint_prepare": [vp],
        "swe_batch_adjoint_prepare": [vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.swe_last_error.restype = ctypes.c_char_p
    L.swe_batch_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def check(status: int, ctx=None, batch: bool = False):
    if status != SWE_OK:
        L = load()
        msg = (L.swe_batch_last_error if batch else L.swe_last_error)(ctx)
        raise SweError(status, msg.decode() if msg else "")
