"""Gradients of gauge-trace losses through the GPU step (discrete adjoint).

``gauge_rollout(w0, z, ...)`` applies a ``torch.autograd.Function``: its
forward runs the taped rollout on the device and returns the surface level at
the gauge cells after every ``obs_every``-th step; its backward runs the
hand-written reverse kernels and returns the gradients with respect to the
initial surface level ``w0`` (per cell) and the node bathymetry ``z`` (per
node).  dt is the forward's CFL step, frozen.  ``batch_gauge_rollout`` is the
same over a batch of independent instances.  Both keep one device context per
mesh across calls (no context creation, precompute or tuning per call), write
a changed bed into it in place, and keep states, traces and gradients in
device memory.
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
        # the adjoint's tables are built with the context, not inside the first taped run
        self.sd._check(_lib.load().swe_adjoint_prepare(self.sd.ctx))

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

    def set_regularisation(self, depth: float) -> None:
        """Depth below which the reverse regularises the slope of a partially
        wet level feeding a node maximum (1e-3 by default; 0 = exact)."""
        self.sd._check(_lib.load().swe_adjoint_set_regularisation(self.sd.ctx, float(depth)))

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
        self.batch._check(_lib.load().swe_batch_adjoint_prepare(self.batch.b))

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

    def set_regularisation(self, depth: float) -> None:
        """As Rollout.set_regularisation, for every instance."""
        self.batch._check(_lib.load().swe_batch_adjoint_set_regularisation(self.batch.b, float(depth)))

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


class _Cache:
    """Contexts kept across autograd calls, one per (mesh objects, flux, cfl),
    least recently used first out."""

    def __init__(self, size: int = 4):
        self.size = size
        self.entries = {}
        self.created = 0

    def get(self, key, make):
        e = self.entries.pop(key, None)
        if e is None:
            e = make()
            self.created += 1
            while len(self.entries) >= self.size:
                self.entries.pop(next(iter(self.entries)))
        self.entries[key] = e
        return e


_CACHE = _Cache()


def cache_info() -> dict:
    """How many contexts the autograd functions created and how many they hold."""
    return {"created": _CACHE.created, "held": len(_CACHE.entries)}


def clear_cache() -> None:
    _CACHE.entries.clear()


def _fluxer_key(fluxer):
    return (fluxer.kind, fluxer.wavespeed) if fluxer is not None else None


class _Entry:
    """A cached context: the meshes it was made for (kept alive, their ids
    are in the key), the node bathymetry it carries now, and a counter of the
    tapes taken on it."""

    def __init__(self, meshes, z0s, holder):
        self.meshes = meshes
        self.z = [np.array(z, dtype=np.float64) for z in z0s]
        self.holder = holder  # a Rollout or a BatchRollout
        self.tape = 0


def _torch_functions():
    import torch

    def _as_dev(t, device):
        return torch.as_tensor(t).detach().to(device=device, dtype=torch.float64).contiguous()

    def _prim_tensor(w0, uv0, device):
        prim = torch.zeros((w0.numel(), 3), dtype=torch.float64, device=device)
        prim[:, 0] = _as_dev(w0, device)
        if uv0 is not None:
            prim[:, 1:] = _as_dev(uv0, device).reshape(-1, 2)
        return prim.contiguous()

    def _device(t):
        return t.device if t.is_cuda else torch.device("cuda", torch.cuda.current_device())

    class GaugeRollout(torch.autograd.Function):
        """(w0 [C], z [N]) -> gauge traces [n_obs, n_gauges] (float64).

        One device context per mesh is created on first use and reused: a new
        bed is written into it in place (swe_set_bathymetry), the initial state
        comes straight from device memory (swe_set_prim_device), and traces and
        gradients stay in device memory (swe_adjoint_*_device)."""

        @staticmethod
        def forward(ctx, w0, z, mesh: Mesh, uv0, gauges, n_steps, obs_every, checkpoint_every, scheme=1, cfl=0.15,
                    fluxer=None):
            device = _device(w0)
            z_np = z.detach().cpu().double().numpy()
            key = ("single", id(mesh), _fluxer_key(fluxer), float(cfl))

            def make():
                geom = mesh.geometry.copy()
                geom[:, 2] = z_np
                m = Mesh(geom, mesh.edge_nodes, mesh.edge_cells, mesh.cell_nodes, mesh.cell_edges,
                         mesh.cell_neighbours)
                return _Entry([mesh], [z_np], Rollout(m, np.zeros((m.num_cells, 3)), fluxer=fluxer, cfl=cfl))

            ent = _CACHE.get(key, make)
            g = np.ascontiguousarray(gauges, dtype=np.int64)
            args = (int(scheme), int(n_steps), int(checkpoint_every), g, int(obs_every))
            traces = GaugeRollout._tape(ent, w0, z_np, uv0, device, args)
            ctx.entry, ctx.args, ctx.device, ctx.tape = ent, args, device, ent.tape
            ctx.inputs = (_as_dev(w0, device), z_np.copy(), uv0)
            return traces

        @staticmethod
        def _tape(ent, w0, z_np, uv0, device, args):
            scheme, n_steps, ckpt, g, obs = args
            sd = ent.holder.sd
            sd.set_stream(torch.cuda.current_stream(device).cuda_stream)
            if not np.array_equal(ent.z[0], z_np):
                sd.set_bathymetry(z_np)
                ent.z[0] = z_np.copy()
            prim = _prim_tensor(w0, uv0, device)
            sd.set_prim_device(prim.data_ptr())
            sd.prime()
            traces = torch.empty((n_steps // obs, len(g)), dtype=torch.float64, device=device)
            sd._check(_lib.load().swe_adjoint_forward_device(sd.ctx, scheme, n_steps, ckpt, len(g), g.ctypes.data,
                                                            obs, ctypes.c_void_p(traces.data_ptr())))
            ent.tape += 1
            return traces

        @staticmethod
        def backward(ctx, grad_traces):
            ent = ctx.entry
            if ent.tape != ctx.tape:
                # another forward ran on this context since: tape this one again
                w0, z_np, uv0 = ctx.inputs
                GaugeRollout._tape(ent, w0, z_np, uv0, ctx.device, ctx.args)
                ctx.tape = ent.tape
            sd = ent.holder.sd
            tg = grad_traces.detach().to(device=ctx.device, dtype=torch.float64).contiguous()
            gp = torch.empty((sd.num_cells, 3), dtype=torch.float64, device=ctx.device)
            gz = torch.empty((sd.num_nodes,), dtype=torch.float64, device=ctx.device)
            sd._check(_lib.load().swe_adjoint_backward_device(sd.ctx, ctypes.c_void_p(tg.data_ptr()),
                                                             ctypes.c_void_p(gp.data_ptr()),
                                                             ctypes.c_void_p(gz.data_ptr())))
            return gp[:, 0].contiguous(), gz, None, None, None, None, None, None, None, None, None

    class BatchGaugeRollout(torch.autograd.Function):
        """Batched form: (w0 [sum C_q], z [sum N_q]) -> traces [n_obs, sum of
        the instances' gauge counts], instances concatenated in order; each
        instance keeps its own CFL dt.  One batch context per tuple of meshes,
        reused like GaugeRollout's."""

        @staticmethod
        def forward(ctx, w0, z, meshes, uv0s, gauges, n_steps, obs_every, checkpoint_every, scheme=1, cfl=0.15,
                    fluxer=None):
            device = _device(w0)
            z_np = z.detach().cpu().double().numpy()
            noff = np.concatenate([[0], np.cumsum([m.num_nodes for m in meshes])]).astype(np.int64)
            zs = [z_np[noff[q]:noff[q + 1]] for q in range(len(meshes))]
            key = ("batch", tuple(id(m) for m in meshes), _fluxer_key(fluxer), float(cfl))

            def make():
                ms, ps = [], []
                for m, zq in zip(meshes, zs):
                    geom = m.geometry.copy()
                    geom[:, 2] = zq
                    ms.append(Mesh(geom, m.edge_nodes, m.edge_cells, m.cell_nodes, m.cell_edges,
                                   m.cell_neighbours))
                    ps.append(np.zeros((m.num_cells, 3)))
                return _Entry(list(meshes), zs, BatchRollout(ms, ps, fluxer=fluxer, cfl=cfl))

            ent = _CACHE.get(key, make)
            coff = ent.holder.cell_off
            g = np.ascontiguousarray(np.concatenate([np.asarray(gq, dtype=np.int64) + coff[q]
                                                     for q, gq in enumerate(gauges)]), dtype=np.int64)
            args = (int(scheme), int(n_steps), int(checkpoint_every), g, int(obs_every))
            traces = BatchGaugeRollout._tape(ent, w0, zs, uv0s, device, args)
            ctx.entry, ctx.args, ctx.device, ctx.tape = ent, args, device, ent.tape
            ctx.inputs = (_as_dev(w0, device), [zq.copy() for zq in zs], uv0s)
            return traces

        @staticmethod
        def _tape(ent, w0, zs, uv0s, device, args):
            scheme, n_steps, ckpt, g, obs = args
            br = ent.holder
            b = br.batch
            b.set_stream(torch.cuda.current_stream(device).cuda_stream)
            changed = [None if np.array_equal(ent.z[q], zs[q]) else zs[q] for q in range(len(zs))]
            if any(c is not None for c in changed):
                b.set_bathymetry(changed)
                for q, c in enumerate(changed):
                    if c is not None:
                        ent.z[q] = c.copy()
            uv = None
            if uv0s is not None:
                uv = np.concatenate([np.asarray(u, dtype=np.float64).reshape(-1, 2) for u in uv0s])
            prim = _prim_tensor(w0, uv, device)
            for q in range(len(zs)):
                b.set_prim_device(q, prim.data_ptr() + 24 * int(br.cell_off[q]))
            b.prime()
            traces = torch.empty((n_steps // obs, len(g)), dtype=torch.float64, device=device)
            b._check(_lib.load().swe_batch_adjoint_forward_device(b.b, scheme, n_steps, ckpt, len(g), g.ctypes.data,
                                                                  obs, ctypes.c_void_p(traces.data_ptr())))
            ent.tape += 1
            return traces

        @staticmethod
        def backward(ctx, grad_traces):
            ent = ctx.entry
            if ent.tape != ctx.tape:
                w0, zs, uv0s = ctx.inputs
                BatchGaugeRollout._tape(ent, w0, zs, uv0s, ctx.device, ctx.args)
                ctx.tape = ent.tape
            br = ent.holder
            tg = grad_traces.detach().to(device=ctx.device, dtype=torch.float64).contiguous()
            gp = torch.empty((int(br.cell_off[-1]), 3), dtype=torch.float64, device=ctx.device)
            gz = torch.empty((int(br.node_off[-1]),), dtype=torch.float64, device=ctx.device)
            br.batch._check(_lib.load().swe_batch_adjoint_backward_device(br.batch.b, ctypes.c_void_p(tg.data_ptr()),
                                                                          ctypes.c_void_p(gp.data_ptr()),
                                                                          ctypes.c_void_p(gz.data_ptr())))
            return gp[:, 0].contiguous(), gz, None, None, None, None, None, None, None, None, None

    return GaugeRollout, BatchGaugeRollout


_FUNCS = None


def _funcs():
    global _FUNCS
    if _FUNCS is None:
        _FUNCS = _torch_functions()
    return _FUNCS


def gauge_rollout(w0, z, mesh: Mesh, gauges, n_steps: int, obs_every: int, checkpoint_every: int, uv0=None,
                  scheme: int = 1, cfl: float = 0.15, fluxer=None):
    """Differentiable gauge traces (torch tensors in, torch tensor out)."""
    return _funcs()[0].apply(w0, z, mesh, uv0, gauges, n_steps, obs_every, checkpoint_every, scheme, cfl, fluxer)


def batch_gauge_rollout(w0, z, meshes, gauges, n_steps: int, obs_every: int, checkpoint_every: int, uv0s=None,
                        scheme: int = 1, cfl: float = 0.15, fluxer=None):
    """Differentiable gauge traces of a batch: w0 / z are the instances'
    initial levels / node bathymetry concatenated in order; gauges is one array
    of local cell ids per instance; returns [n_obs, sum of gauge counts]."""
    return _funcs()[1].apply(w0, z, tuple(meshes), uv0s, gauges, n_steps, obs_every, checkpoint_every, scheme, cfl,
                             fluxer)
