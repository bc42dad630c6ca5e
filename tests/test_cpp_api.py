"""The reference's C++ API over the C ABI (include/swe_fvm_gb300.hpp): the
header compiles, a driver written against it links, rejects a bad mesh with
DomainError before touching the device (no GPU needed), and on the GPU gives
the Python API's state bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from swe_fvm_gb300 import Fluxes, SpaceDisc, TimeDisc, Solvers, Wavespeeds, scenarios
from swe_fvm_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "reference_api_main.cpp")


def _cuda_lib_dir():
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib", "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return "/usr/local/cuda/lib64"


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    lib = build()
    out = str(tmp_path_factory.mktemp("cpp") / "reference_api_main")
    libdir = os.path.dirname(lib)
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        SRC, "-o", out, "-L", libdir, "-lswe_gb300", "-L", _cuda_lib_dir(), "-lcudart",
                        f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{_cuda_lib_dir()}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _write(path, m, prim, steps):
    m = m.contiguous()
    with open(path, "wb") as f:
        np.array([m.num_nodes, m.num_edges, m.num_cells, steps], dtype=np.int64).tofile(f)
        np.ascontiguousarray(m.geometry, dtype=np.float64).tofile(f)
        for a in (m.edge_nodes, m.edge_cells, m.cell_nodes, m.cell_edges, m.cell_neighbours):
            np.ascontiguousarray(a, dtype=np.int64).tofile(f)
        np.ascontiguousarray(prim, dtype=np.float64).tofile(f)


def assigned(m, prim):
    """The field v0.prim(i) = prim[i] leaves: PrimAssigner (src/Assigners.cpp:
    8-20) with the centroid bathymetry, as the restatement computes it."""
    import ctypes

    from oracle.oracle import lib as oracle_lib

    L = oracle_lib()
    bc = m.centroids()[:, 2]
    out = np.empty_like(prim)
    tmp_in, tmp_out = np.empty(3), np.empty(3)
    for i in range(m.num_cells):
        tmp_in[:] = prim[i]
        L.oracle_prim_assign(float(bc[i]), tmp_in.ctypes.data_as(ctypes.c_void_p),
                             tmp_out.ctypes.data_as(ctypes.c_void_p))
        out[i] = tmp_out
    return out


def test_volume_field_assigners_on_the_host(driver, tmp_path):
    """The VolumeField written through prim(i) equals the restatement's
    PrimAssigner cell by cell (thin films, dry cells, velocities), with no GPU:
    the driver fails only when it reaches the device."""
    m, prim = scenarios.random_front_case(30, 7)
    _write(tmp_path / "in.bin", m, prim, 0)
    r = subprocess.run([driver, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True)
    if r.returncode == 0:
        raw = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
        assert np.array_equal(raw[:3 * m.num_cells].reshape(-1, 3), assigned(m, prim))
    else:
        pytest.skip("no device here: the field is checked by the GPU test")


def test_driver_rejects_a_bad_mesh_with_domain_error(driver, tmp_path):
    m, prim = scenarios.lake_at_rest(4)
    m = m.contiguous()
    m.edge_cells = m.edge_cells.copy()
    m.edge_cells[np.argmax(m.edge_cells[:, 1] < 0), 1] = -2
    _write(tmp_path / "in.bin", m, prim, 1)
    r = subprocess.run([driver, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True)
    assert r.returncode == 2 and "DomainError" in r.stderr, (r.returncode, r.stderr)


@pytest.mark.gpu
def test_driver_equals_the_python_api(gpu, driver, tmp_path):
    m, prim = scenarios.random_front_case(30, 7)
    n = 12
    _write(tmp_path / "in.bin", m, prim, n)
    r = subprocess.run([driver, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
    C = m.num_cells
    v0, got, t = raw[:3 * C].reshape(-1, 3), raw[3 * C:-1].reshape(-1, 3), raw[-1]
    assert np.array_equal(v0, assigned(m, prim))
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, v0)
    td = TimeDisc(sd)
    t_py = 0.0
    for _ in range(n):
        dt = td.CFLdt()
        Solvers.SSPRK2(td, dt)
        t_py += dt
    assert np.array_equal(got, sd.GetVolField())
    assert t == t_py
