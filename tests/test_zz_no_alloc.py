"""The allocation-free edge-flux pass against the context's own flux pass.

swe_edge_fluxes_noalloc exists for callers that cannot call cudaMalloc (a
framework that owns device memory through its own pool, a real-time loop, a
plugin handed only device pointers): they pass inputs and outputs, and the
pass keeps its scratch in a fixed static device array.  Here the edge
geometry is computed on the host with the reference's formulas
(src/Bathymetry.cpp:69-90, include/Fluxes.h:43-44), the interface states come
from a context's SpaceDisc::ComputeInterfaceValues, and two calls in a row
must reproduce the context's fluxes and CFL ratio (same tolerance as the
other parity tests).
"""
import ctypes

import numpy as np
import pytest

from swe_fvm_gb300 import Fluxes, SpaceDisc, Wavespeeds, _lib, scenarios
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


def edge_geometry(m):
    g = m.geometry
    en, ec = m.edge_nodes, m.edge_cells
    p0, p1 = g[en[:, 0]], g[en[:, 1]]
    L = np.sqrt((p0[:, 0] - p1[:, 0]) * (p0[:, 0] - p1[:, 0]) + (p0[:, 1] - p1[:, 1]) * (p0[:, 1] - p1[:, 1]))
    k = 1.0 / 3.0
    cp = g[m.cell_nodes]
    T = cp[:, 0] * k + cp[:, 1] * k + cp[:, 2] * k
    ba = cp[:, 1, :2] - cp[:, 0, :2]
    ca = cp[:, 2, :2] - cp[:, 0, :2]
    A = 0.5 * np.abs(ba[:, 0] * ca[:, 1] - ca[:, 0] * ba[:, 1])
    o = ec[:, 0]
    t0 = (p1[:, 0] - p0[:, 0]) / L
    t1 = (p1[:, 1] - p0[:, 1]) / L
    d0 = T[o, 0] - p0[:, 0]
    d1 = T[o, 1] - p0[:, 1]
    flip = d0 * t1 - t0 * d1 > 0.0
    t0 = np.where(flip, -t0, t0)
    t1 = np.where(flip, -t1, t1)
    b = (p0[:, 2] + p1[:, 2]) * 0.5
    nb = np.where(ec[:, 1] < 0, o, ec[:, 1])
    dl = 2.0 * A[o] / L
    dr = 2.0 * A[nb] / L
    lmin = np.where(dr < dl, dr, dl)
    return np.ascontiguousarray(np.stack([t1, -t0, t0, t1, b, lmin], axis=1))


def _run_case(m, prim, flux, ws):
    import torch

    fluxer = Fluxes.HLLC(ws) if flux == 1 else Fluxes.HLL(ws)
    sd = SpaceDisc(fluxer, m, prim)
    sd.ComputeInterfaceValues()
    sd.ComputeFluxes()
    f_ref = sd.GetFluxes()
    r_ref = sd.GetMinLenToWavespeed()
    edg = sd.GetEdgField()
    ec = m.edge_cells
    interior = np.where(ec[:, 1] >= 0)[0]
    o, n = ec[interior, 0], ec[interior, 1]
    left = edg[2 * interior + (o < n)]
    right = edg[2 * interior + (n < o)]
    geom = edge_geometry(m)[interior]
    dev = torch.device("cuda", 0)
    d_geom = torch.from_numpy(geom).to(dev)
    d_left = torch.from_numpy(np.ascontiguousarray(left)).to(dev)
    d_right = torch.from_numpy(np.ascontiguousarray(right)).to(dev)
    d_flux = torch.full((len(interior), 3), float("nan"), dtype=torch.float64, device=dev)
    d_ratio = torch.zeros(1, dtype=torch.float64, device=dev)
    L = _lib.load()
    free = []
    for call in range(2):
        d_flux.fill_(float("nan"))
        d_ratio.fill_(-1.0)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        st = L.swe_edge_fluxes_noalloc(flux, ws, len(interior), d_geom.data_ptr(), d_left.data_ptr(),
                                       d_right.data_ptr(), 0.0, d_flux.data_ptr(), d_ratio.data_ptr(), None)
        assert st == 0
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        f = d_flux.cpu().numpy()
        assert rel_l2(f, f_ref[interior]) <= TOL, call
        assert float(d_ratio.item()) == pytest.approx(r_ref, rel=TOL), call
    # the second call (after the first has loaded the module into this
    # context) leaves the device's free memory exactly as it found it
    assert free[3] == free[2]
    return len(interior)


@pytest.mark.parametrize("flux,ws", [(1, 2), (0, 2), (1, 0)])
def test_noalloc_flux_pass_matches_context(gpu, flux, ws):
    m, prim = scenarios.random_front_case(40, seed=11)
    _run_case(m, prim, flux, ws)


def test_noalloc_many_blocks_matches_context(gpu):
    """More than 256 blocks of partial minima (over 65,536 interior edges), so
    every thread of the folding block reads several partial minima."""
    m, prim = scenarios.random_front_case(200, seed=5)
    n = _run_case(m, prim, 1, 2)
    assert n > 65536


def test_noalloc_rejects_sizes_beyond_the_scratch(gpu):
    L = _lib.load()
    x = ctypes.c_double()
    assert L.swe_edge_fluxes_noalloc(1, 2, 16777217, 1, 1, 1, 0.0, 1, ctypes.addressof(x), None) == 1
    assert L.swe_edge_fluxes_noalloc(1, 2, 0, 1, 1, 1, 0.0, 1, ctypes.addressof(x), None) == 1
