"""Gradients of gauge-trace losses through the GPU step (discrete adjoint).

``GaugeRollout.apply(w0, z, ...)`` is a ``torch.autograd.Function``: its
forward runs the taped rollout on the device (swe_adjoint_forward) and returns
the surface level at the gauge cells after every ``obs_every``-th step; its
backward runs the hand-written reverse kernels (swe_adjoint_backward) and
returns the gradients with respect to the initial surface level ``w0`` (per
cell) and the node bathymetry ``z`` (per node).  dt is the forward's CFL step,
frozen.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .mesh import Mesh
from .solver import Batch, Fluxes, SpaceDisc, Wavespeeds


class Rollout:
    """A taped forward run and its adjoint, without PyTorch."""

    def __init__(self, mesh: Mesh, prim0, fluxer=None, cfl=0.15, cor=0.0, reorder="auto", block=0):
        self.mesh = mesh.contiguous()
        self.sd = SpaceDisc(fluxer or Fluxes.HLLC(Wavespeeds.Einfeldt), self.mesh, prim0, cor=cor, cfl=cfl,
                            reorder=reorder, block=block)

    def forward(self, scheme: int, n_steps: int, checkpoint_every: int, gauges, obs_every: int) -> np.ndarray:
        g = np.ascontiguousarray(gauges, dtype=np.int64)
        n_obs = n_steps // obs_every
        traces = np.zeros((n_obs, len(g)))
        L = _lib.load()
        self.sd._check(L.swe_adjoint_forward(self.sd.ctx, int(scheme), int(n_steps), int(checkpoint_every), len(g),
                                             g.ctypes.data, int(obs_every), traces.ctypes.data))
        return traces

    def dts(self, n_steps: int) -> np.ndarray:
        out = np.zeros(n_steps)
        self.sd._check(_lib.load().swe_adjoint_dts(self.sd.ctx, out.ctypes.data))
        return out

    def backward(self, trace_grads):
        tg = np.ascontiguousarray(trace_grads, dtype=np.float64)
        gp = np.zeros((self.mesh.num_cells, 3))
        gz = np.zeros(self.mesh.num_nodes)
        L = _lib.load()
        self.sd._check(L.swe_adjoint_backward(self.sd.ctx, tg.ctypes.data, gp.ctypes.data, gz.ctypes.data))
        return gp, gz


class BatchRollout:
    """The taped forward run and its adjoint for a batch of independent
    instances: one launch per stage kernel over all of them, each instance with
    its own CFL dt, gauges and gradients."""

    def __init__(self, meshes, prims, fluxer=None, cfl=0.15, cor=0.0, reorder="auto", block=0):
        self.meshes = [m.contiguous() for m in meshes]
        self.batch = Batch(self.meshes, prims, fluxer=fluxer, cor=cor, cfl=cfl, reorder=reorder, block=block)
        self.cell_off = np.concatenate([[0], np.cumsum([m.num_cells for m in self.meshes])]).astype(np.int64)
        self.node_off = np.concatenate([[0], np.cumsum([m.num_nodes for m in self.meshes])]).astype(np.int64)
        self.gauge_counts = []

    def forward(self, scheme: int, n_steps: int, checkpoint_every: int, gauges, obs_every: int):
        """gauges: one array of local cell ids per instance.  Returns one
        (n_steps // obs_every, n_gauges_q) trace array per instance."""
        self.gauge_counts = [len(gq) for gq in gauges]
        g = np.concatenate([np.asarray(gq, dtype=np.int64) + self.cell_off[q] for q, gq in enumerate(gauges)])
        g = np.ascontiguousarray(g, dtype=np.int64)
        n_obs = n_steps // obs_every
        traces = np.zeros((n_obs, len(g)))
        self.batch._check(_lib.load().swe_batch_adjoint_forward(self.batch.b, int(scheme), int(n_steps),
                                                                int(checkpoint_every), len(g), g.ctypes.data,
                                                                int(obs_every), traces.ctypes.data))
        cut = np.cumsum([0] + self.gauge_counts)
        return [traces[:, cut[q]:cut[q + 1]] for q in range(len(self.meshes))]

    def dts(self, n_steps: int) -> np.ndarray:
        """(n_steps, n_instances) recorded dts."""
        out = np.zeros((n_steps, len(self.meshes)))
        self.batch._check(_lib.load().swe_batch_adjoint_dts(self.batch.b, out.ctypes.data))
        return out

    def backward(self, trace_grads):
        """trace_grads: one array per instance, shaped like its traces.
        Returns one (grad_prim0 (C_q, 3), grad_z (N_q,)) pair per instance."""
        tg = np.ascontiguousarray(np.concatenate([np.asarray(t, dtype=np.float64) for t in trace_grads], axis=1))
        gp = np.zeros((int(self.cell_off[-1]), 3))
        gz = np.zeros(int(self.node_off[-1]))
        self.batch._check(_lib.load().swe_batch_adjoint_backward(self.batch.b, tg.ctypes.data, gp.ctypes.data,
                                                                 gz.ctypes.data))
        return [(gp[self.cell_off[q]:self.cell_off[q + 1]], gz[self.node_off[q]:self.node_off[q + 1]])
                for q in range(len(self.meshes))]


def _torch_function():
    import torch

    class GaugeRollout(torch.autograd.Function):
        """(w0 [C], z [N]) -> gauge traces [n_obs, n_gauges] (float64)."""

        @staticmethod
        def forward(ctx, w0, z, mesh: Mesh, uv0, gauges, n_steps, obs_every, checkpoint_every, scheme=1, cfl=0.15,
                    fluxer=None):
            geom = mesh.geometry.copy()
            geom[:, 2] = z.detach().cpu().double().numpy()
            m = Mesh(geom, mesh.edge_nodes, mesh.edge_cells, mesh.cell_nodes, mesh.cell_edges, mesh.cell_neighbours)
            prim = np.zeros((m.num_cells, 3))
            prim[:, 0] = w0.detach().cpu().double().numpy()
            if uv0 is not None:
                prim[:, 1:] = np.asarray(uv0, dtype=np.float64)
            ro = Rollout(m, prim, fluxer=fluxer, cfl=cfl)
            traces = ro.forward(scheme, n_steps, checkpoint_every, gauges, obs_every)
            ctx.rollout = ro
            ctx.device = w0.device
            return torch.from_numpy(traces).to(w0.device)

        @staticmethod
        def backward(ctx, grad_traces):
            gp, gz = ctx.rollout.backward(grad_traces.detach().cpu().double().numpy())
            gw = torch.from_numpy(gp[:, 0].copy()).to(ctx.device)
            gzt = torch.from_numpy(gz).to(ctx.device)
            return gw, gzt, None, None, None, None, None, None, None, None, None

    return GaugeRollout


_GR = None


def gauge_rollout(w0, z, mesh: Mesh, gauges, n_steps: int, obs_every: int, checkpoint_every: int, uv0=None,
                  scheme: int = 1, cfl: float = 0.15, fluxer=None):
    """Differentiable gauge traces (torch tensors in, torch tensor out)."""
    global _GR
    if _GR is None:
        _GR = _torch_function()
    return _GR.apply(w0, z, mesh, uv0, gauges, n_steps, obs_every, checkpoint_every, scheme, cfl, fluxer)
