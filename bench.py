"""Benchmark: FP64 cell-updates/s of the explicit finite-volume step on 1 GB300.

Workload (single large unstructured mesh): Delaunay triangulation of a
708 x 708 seeded jittered lattice on the unit square (about 1.0M triangles),
Morton-ordered; bed = 8 Gaussian bumps (heights U[0.05,0.3], widths
U[0.02,0.1]) over a flat floor at 0; surface 0.5 for x < 0.3 else 0.2, raised
to the bed where bumps emerge; HLLC + Einfeldt; SSPRK2; dt = CFLdt() with the
reference's coefficient 0.15 before every step.  A "step" is one full SSPRK2
step (2 stages: reconstruction, fluxes with the CFL reduction, update) of the
whole mesh.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  value = cells x steps / device time of K steps replayed
from a CUDA graph with the state resident in HBM; e2e = the same through the
C ABI with host buffers (swe_set_prim + swe_step + swe_get_prim per step, the
copies inside the timed region).  --impl reference times the CPU restatement
of the reference solver on the host cores instead.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# Compulsory HBM bytes of one ideally fused SSPRK2 cell-step (FP64 state, int32
# connectivity): per stage read prim 24 + write prim 24 + 6 ids 24 + node xyz
# 24 x N/C ~ 12 = 84 B; stage 2 re-reads the step's initial state, 24 B.
BYTES_PER_CELL_STEP = 2 * 84 + 24
# FP64 instructions issued per SSPRK2 cell-step by the step kernels: ncu
# smsp__sass_thread_inst_executed_op_fp64_pred_on summed over the 12 launches
# of one step of the dam break at lattice 500 (498,002 cells): 1.942e8, i.e.
# per stage k_flux 62 per edge x 1.5 edges per cell + k_update 73-79 +
# k_recon1 18 + k_drain 7 per cell, plus the few part-wet cells.  The bound of
# the step on GB300, whose FP64 pipe issues one instruction per lane and cycle
# (DFMA = 2 flops).
FP64_INST_PER_CELL_STEP = 390
LATTICE = int(os.environ.get("SWE_BENCH_LATTICE", "708"))
CFL = 0.15


def workload():
    from swe_fvm_gb300 import scenarios

    t0 = time.time()
    mesh, prim = scenarios.dam_break(lattice=LATTICE)
    return mesh, prim, time.time() - t0


def workload_config(mesh, world):
    """The workload both arms run (the same dict in the GPU line and the
    reference line)."""
    return {"workload": "dam_break_1M", "cells": mesh.num_cells, "edges": mesh.num_edges, "nodes": mesh.num_nodes,
            "flux": "HLLC+Einfeldt", "scheme": "SSPRK2", "cfl": CFL, "dt": "CFLdt() per step",
            "l2": "working set > 1 GB, larger than the 129 MB L2; no flush", "parallelism": f"replicas x{world}"}


def run_thacker(torch, stream, steps: int = 1000):
    """Workload: Thacker bowl on [-2,2]^2, 64 x 64 squares x 2 triangles (8192
    cells), HLLC + Einfeldt, SSPRK2, CFL 0.4, 1000 steps with dt from the
    device CFL reduction (graph-replayed), beside the single-thread CPU
    restatement on the same run.  The GPU run's states equal the reference's
    own solver bit for bit (tests/test_gpu_ref_golden.py)."""
    from oracle.oracle import Oracle
    from swe_fvm_gb300 import Fluxes, SpaceDisc, Wavespeeds, scenarios

    m, prim = scenarios.thacker(64)
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, prim, cfl=0.4)
    sd.set_stream(stream.cuda_stream)
    sd.ComputeInterfaceValues()
    sd.ComputeFluxes()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    t_end = sd.run_cfl(1, steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    o = Oracle(m, prim)
    o.compute_interface_values()
    o.compute_fluxes()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step("SSPRK2", 0.4 * o.min_len_to_wavespeed())
    cpu_s = time.perf_counter() - t0
    return {"metric": "cell-updates/s (Thacker 64x64x2, SSPRK2, CFL 0.4, 1000 steps)",
            "value": m.num_cells * steps / (ms * 1e-3), "unit": "cell-updates/s", "ms_per_step": ms / steps,
            "steps": steps, "simulated_time": t_end,
            "note": "first 1000 steps from a fresh context, including the graph capture of the first replay",
            "cpu_restatement_1_thread": m.num_cells * steps / cpu_s}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once sampling is live
            t0 = time.time()
            while not self.rows and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[3:]) if v.strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline(mesh, prim, budget_s: float = 10.0):
    """The single-threaded CPU restatement on a bounded sample of the same workload."""
    from oracle.oracle import Oracle

    o = Oracle(mesh, prim)
    o.compute_interface_values()
    o.compute_fluxes()
    t0 = time.perf_counter()
    o.step("SSPRK2", CFL * o.min_len_to_wavespeed())
    t1 = time.perf_counter() - t0
    n_more = max(0, min(30, int(budget_s / max(t1, 1e-9)) - 1))
    t0 = time.perf_counter()
    for _ in range(n_more):
        o.step("SSPRK2", CFL * o.min_len_to_wavespeed())
    t = t1 + (time.perf_counter() - t0)
    n = 1 + n_more
    return {"value": mesh.num_cells * n / t, "unit": "cell-updates/s", "cores": 1, "kind": "port",
            "sample": f"{n} SSPRK2 steps of the full {mesh.num_cells}-cell mesh, single thread, {t:.1f} s"}


def dist_setup(n_gpus):
    """Replicas only: one process per GPU, no collective on the data path.
    NCCL on GPUs; gloo when no GPU is visible (the CPU tests of this logic)."""
    import torch

    if n_gpus > 1 or "WORLD_SIZE" in os.environ:
        import torch.distributed as dist

        local = int(os.environ.get("LOCAL_RANK", "0"))
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        return dist, dist.get_rank(), dist.get_world_size(), local
    return None, 0, 1, 0


def max_over_ranks(ms, dist):
    """The slowest rank's time (the whole job's time for weak-scaled replicas)."""
    if not dist:
        return ms
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def job_rate(world, cells, steps, ms):
    """Whole-job cell-updates/s: every rank advanced its own replica."""
    return world * cells * steps / (ms * 1e-3)


def run_gpu(args):
    import torch

    from swe_fvm_gb300 import Fluxes, SpaceDisc, TimeDisc, Wavespeeds, _lib

    dist, rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    if args.ensemble_profile:
        # profiling driver for the batched form: the 256-instance ensemble,
        # warm-up, then exactly K graph-replayed steps inside the profiled range
        from swe_fvm_gb300 import Batch, Fluxes, Wavespeeds, scenarios

        ens = scenarios.ensemble(ENSEMBLE_INSTANCES)
        b = Batch([e[0] for e in ens], [e[1] for e in ens], Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.4)
        b.run_cfl(1, args.warmup)
        b.synchronize()
        torch.cuda.cudart().cudaProfilerStart()
        b.run_cfl(1, args.steps)
        b.synchronize()
        torch.cuda.cudart().cudaProfilerStop()
        print(json.dumps({"ensemble_profile": True, "instances": len(ens),
                          "cells": int(sum(e[0].num_cells for e in ens)), "steps": args.steps,
                          "tuning": b.tuning(0)}))
        return
    if args.thacker_profile:
        # profiling driver for the small-mesh configuration: the 8192-cell
        # Thacker bowl (CFL 0.4), warm-up, then exactly K graph-replayed steps
        # inside the profiled range
        from swe_fvm_gb300 import scenarios

        tm, tp = scenarios.thacker(64)
        ts = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), tm, tp, cfl=0.4)
        ts.run_cfl(1, args.warmup)
        ts.synchronize()
        torch.cuda.cudart().cudaProfilerStart()
        ts.run_cfl(1, args.steps)
        ts.synchronize()
        torch.cuda.cudart().cudaProfilerStop()
        print(json.dumps({"thacker_profile": True, "cells": tm.num_cells, "steps": args.steps,
                          "tuning": ts.tuning()}))
        return
    mesh, prim, t_gen = workload()
    C = mesh.num_cells
    sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), mesh, prim, cfl=CFL)
    # a dedicated stream: the library's kernels and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sd.set_stream(stream.cuda_stream)
    if args.adjoint_profile:
        # profiling driver for the reverse kernels: the adjoint workload's mesh,
        # a short plain run, a short taped run and its reverse, wall-timed
        from swe_fvm_gb300 import scenarios
        from swe_fvm_gb300.adjoint import Rollout

        am, ap = scenarios.hump_instance(2024, ADJ_CELLS)
        am = am.contiguous()
        gauges = np.random.default_rng(11).choice(am.num_cells, 64, replace=False)
        ps = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), am, ap)
        ps.set_stream(stream.cuda_stream)
        ro = Rollout(am, ap)
        torch.cuda.synchronize()
        # the profiled range (ncu --profile-from-start off): creation and
        # tuning stay outside it
        torch.cuda.cudart().cudaProfilerStart()
        ps.run_cfl(1, 2)
        ps.synchronize()
        t0 = time.perf_counter()
        ps.run_cfl(1, args.steps)
        ps.synchronize()
        t_plain = time.perf_counter() - t0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tr = ro.forward(1, args.steps, 50, gauges, 10)
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        ro.backward(np.ones_like(tr))
        t_bwd = time.perf_counter() - t0
        torch.cuda.cudart().cudaProfilerStop()
        print(json.dumps({"adjoint_profile": True, "cells": am.num_cells, "steps": args.steps,
                          "plain_s": t_plain, "taped_forward_s": t_fwd, "backward_s": t_bwd,
                          "ratio": (t_fwd + t_bwd) / t_plain}))
        return
    if args.profile:
        # profiling driver: warm-up, then exactly K graph-replayed steps inside
        # the profiled range (ncu --profile-from-start off)
        sd.run_cfl(1, args.warmup)
        sd.synchronize()
        torch.cuda.cudart().cudaProfilerStart()
        sd.run_cfl(1, args.steps)
        sd.synchronize()
        torch.cuda.cudart().cudaProfilerStop()
        print(json.dumps({"profile": True, "cells": C, "steps": args.steps, "warmup": args.warmup}))
        return
    # warm-up (graph capture happens on the first replay)
    sd.run_cfl(1, args.warmup)
    torch.cuda.synchronize()
    n0 = sd.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        _lib.check(_lib.load().swe_run_cfl(sd.ctx, 1, args.steps, None), sd.ctx)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    launches = sd.launch_count() - n0
    ms = max_over_ranks(ms, dist)
    sd.synchronize()
    value = job_rate(world, C, args.steps, ms)
    ms_step = ms / args.steps

    # per-kernel CUDA-event timings (kernel by kernel, same stream)
    kt = sd.time_kernels(1, 3)
    names = ["recon_pass1", "recon_pass2", "flux", "draining_dt", "update"]
    per = {n: float(v) for n, v in zip(names, kt[:5])}

    # end to end through the C ABI with host buffers
    pinned = torch.empty((C, 3), dtype=torch.float64, pin_memory=True)
    host = pinned.numpy()
    host[:] = sd.GetVolField()
    L = _lib.load()
    dt = TimeDisc(sd).CFLdt()
    n_e2e = max(3, min(args.steps, 20))
    for _ in range(2):
        L.swe_set_prim(sd.ctx, host.ctypes.data)
        L.swe_step(sd.ctx, 1, dt)
        L.swe_get_prim(sd.ctx, host.ctypes.data)
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        _lib.check(L.swe_set_prim(sd.ctx, host.ctypes.data), sd.ctx)
        _lib.check(L.swe_step(sd.ctx, 1, dt), sd.ctx)
        _lib.check(L.swe_get_prim(sd.ctx, host.ctypes.data), sd.ctx)
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * C * n_e2e / e2e_s, "unit": "cell-updates/s", "h2d_bytes_per_step": 24 * C,
           "d2h_bytes_per_step": 24 * C, "steps": n_e2e,
           "api": "swe_set_prim + swe_step + swe_get_prim (pinned host buffers)"}

    # the same workload with the HLL plugin (the configuration names HLL and HLLC)
    sd_hll = SpaceDisc(Fluxes.HLL(Wavespeeds.Einfeldt), mesh, prim, cfl=CFL)
    sd_hll.set_stream(stream.cuda_stream)
    sd_hll.run_cfl(1, args.warmup)
    torch.cuda.synchronize()
    e0.record(stream)
    _lib.check(_lib.load().swe_run_cfl(sd_hll.ctx, 1, args.steps, None), sd_hll.ctx)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_hll = e0.elapsed_time(e1)
    hll = {"value": world * C * args.steps / (ms_hll * 1e-3), "unit": "cell-updates/s",
           "ms_per_step": ms_hll / args.steps, "flux": "HLL+Einfeldt"}
    del sd_hll

    fp64 = ctypes.c_double(0.0)
    _lib.check(L.swe_measure_fp64_peak(ctypes.byref(fp64)))
    hbm, src = peaks()
    achieved = BYTES_PER_CELL_STEP * C / (ms_step * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": "ssprk2_step (one CUDA graph: 2 stages x 6 kernels on two streams)",
            "achieved": achieved,
            "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "peak_source": src,
            "algorithmic_bytes_per_launch": BYTES_PER_CELL_STEP * C,
            "traffic": TRAFFIC_PER_STEP.get(LATTICE),
            "kernel_ms_per_launch": per, "fp64_peak_tflops_measured": fp64.value,
            "fp64_issue": {"inst_per_cell_step": FP64_INST_PER_CELL_STEP,
                           "achieved_tinst_per_s": FP64_INST_PER_CELL_STEP * C / (ms_step * 1e-3) / 1e12,
                           "peak_tinst_per_s": fp64.value / 2,
                           "frac": FP64_INST_PER_CELL_STEP * C / (ms_step * 1e-3) / 1e12 / (fp64.value / 2)}}

    out = {
        "metric": "cell-updates/s (plain FP64 SSPRK2 step, 1M-triangle unstructured mesh)",
        "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded jittered-lattice Delaunay mesh, Gaussian bumps, dam break)",
        "config": workload_config(mesh, world),
        "tuning": sd.tuning(), "mesh_gen_s": round(t_gen, 1),
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "clocks": clk.summary(), "hll": hll,
        "thacker_8192": run_thacker(torch, stream),
    }
    if ENSEMBLE_INSTANCES > 0 and not args.no_ensemble:
        out["batched"] = run_ensemble(torch, stream)
    if ADJ_STEPS > 0 and not args.no_adjoint:
        out["adjoint"] = run_adjoint(torch, stream)
    if BADJ_INSTANCES > 0 and not args.no_batch_adjoint:
        out["batched_adjoint"] = run_batch_adjoint(torch, stream)
    if args.layouts:
        out["layouts"] = run_layouts(torch, stream, mesh, prim, args.steps, args.warmup)
    if rank == 0:
        if world == 1 and not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(mesh, prim)
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def run_layouts(torch, stream, mesh, prim, steps, warmup):
    """Plain SSPRK2 step time of the same mesh in each device order, and of a
    copy numbered at random (caller's order kept vs the tuner's choice)."""
    from swe_fvm_gb300 import Fluxes, SpaceDisc, Wavespeeds, _lib
    from swe_fvm_gb300.mesh import shuffled

    smesh, cf, _, _ = shuffled(mesh, 123)
    sprim = prim[cf]
    cases = [("generated/keep", mesh, prim, "keep"), ("generated/morton", mesh, prim, "morton"),
             ("generated/rcm", mesh, prim, "rcm"), ("generated/auto", mesh, prim, "auto"),
             ("shuffled/keep", smesh, sprim, "keep"), ("shuffled/auto", smesh, sprim, "auto")]
    out = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for label, m, p, reorder in cases:
        t0 = time.perf_counter()
        sd = SpaceDisc(Fluxes.HLLC(Wavespeeds.Einfeldt), m, p, cfl=CFL, reorder=reorder)
        t_create = time.perf_counter() - t0
        sd.set_stream(stream.cuda_stream)
        sd.run_cfl(1, warmup)
        torch.cuda.synchronize()
        e0.record(stream)
        _lib.check(_lib.load().swe_run_cfl(sd.ctx, 1, steps, None), sd.ctx)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        kt = sd.time_kernels(1, 3)
        out[label] = {"ms_per_step": ms, "cell_updates_per_s": m.num_cells / (ms * 1e-3), "tuning": sd.tuning(),
                      "create_s": round(t_create, 2),
                      "kernel_ms": dict(zip(["recon_pass1", "recon_pass2", "flux", "draining_dt", "update"],
                                            [round(float(x), 4) for x in kt[:5]]))}
        del sd
    return out


ENSEMBLE_INSTANCES = int(os.environ.get("SWE_BENCH_ENSEMBLE", "256"))
ENSEMBLE_STEPS = int(os.environ.get("SWE_BENCH_ENSEMBLE_STEPS", "200"))


def run_ensemble(torch, stream):
    """Ensemble config: 256 seeded Delaunay instances, 2k-200k cells
    (log-uniform), HLLC + Einfeldt, SSPRK2, per-instance CFL 0.4, 200 steps.
    Batched: every stage kernel covers all instances (one graph per step).
    Plain: the same instances stepped one after another with the plain step."""
    from swe_fvm_gb300 import Batch, Fluxes, SpaceDisc, Wavespeeds, scenarios

    t0 = time.time()
    ens = scenarios.ensemble(ENSEMBLE_INSTANCES)
    t_gen = time.time() - t0
    meshes = [m for m, _ in ens]
    prims = [p for _, p in ens]
    cells = sum(m.num_cells for m in meshes)
    fl = Fluxes.HLLC(Wavespeeds.Einfeldt)
    K = ENSEMBLE_STEPS
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # batched
    b = Batch(meshes, prims, fl, cfl=0.4)
    b.set_stream(stream.cuda_stream)
    b.run_cfl(1, 3)
    torch.cuda.synchronize()
    n0 = b.launch_count()
    e0.record(stream)
    b.run_cfl(1, K)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_b = e0.elapsed_time(e1)
    launches_b = b.launch_count() - n0
    b.synchronize()
    tuning_b = b.tuning(0)
    del b
    # plain, one instance after another
    sds = []
    for m, p in ens:
        sd = SpaceDisc(fl, m, p, cfl=0.4)
        sd.set_stream(stream.cuda_stream)
        sd.run_cfl(1, 3)
        sds.append(sd)
    torch.cuda.synchronize()
    e0.record(stream)
    for sd in sds:
        sd.run_cfl(1, K)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_p = e0.elapsed_time(e1)
    for sd in sds:
        sd.synchronize()
    del sds
    vb = cells * K / (ms_b * 1e-3)
    vp = cells * K / (ms_p * 1e-3)
    return {"metric": "cell-updates/s (batched FP64 SSPRK2 ensemble)", "value": vb, "unit": "cell-updates/s",
            "plain_sequential_value": vp, "speedup_vs_plain": vb / vp, "instances": len(ens), "cells": cells,
            "steps": K, "ms_per_step": ms_b / K, "plain_ms_per_step": ms_p / K, "gpu_launches": launches_b,
            "config": {"workload": "ensemble_256", "cells_per_instance": "log-uniform 2k-200k", "cfl": 0.4,
                       "flux": "HLLC+Einfeldt", "scheme": "SSPRK2", "mesh_gen_s": round(t_gen, 1),
                       "tuning": tuning_b}}


ADJ_CELLS = int(os.environ.get("SWE_BENCH_ADJ_CELLS", "250000"))
ADJ_STEPS = int(os.environ.get("SWE_BENCH_ADJ_STEPS", "2000"))


def run_adjoint(torch, stream):
    """Adjoint config: 250k-cell seeded Delaunay mesh, bump bathymetry, hump
    surface, SSPRK2 (HLLC + Einfeldt, CFL 0.15), 2000 steps, 64 random gauge
    cells observed every 10th step, checkpoint every 50 steps; target traces
    from a run whose bathymetry carries 5% seeded Gaussian noise.  Reports the
    cost ratio (taped forward + backward) / plain forward solve and runs the
    loss gradient once through the torch.autograd.Function."""
    from swe_fvm_gb300 import Fluxes, SpaceDisc, Wavespeeds, scenarios
    from swe_fvm_gb300.adjoint import Rollout, gauge_rollout
    from swe_fvm_gb300.mesh import Mesh

    mesh, prim = scenarios.hump_instance(2024, ADJ_CELLS)
    mesh = mesh.contiguous()
    rng = np.random.default_rng(11)
    gauges = rng.choice(mesh.num_cells, 64, replace=False)
    obs, ckpt = 10, 50
    g = mesh.geometry.copy()
    g[:, 2] = g[:, 2] * (1.0 + 0.05 * rng.standard_normal(mesh.num_nodes))
    noisy = Mesh(g, mesh.edge_nodes, mesh.edge_cells, mesh.cell_nodes, mesh.cell_edges, mesh.cell_neighbours)
    target = Rollout(noisy, prim).forward(1, ADJ_STEPS, ckpt, gauges, obs)
    fl = Fluxes.HLLC(Wavespeeds.Einfeldt)
    # plain forward solve
    sd = SpaceDisc(fl, mesh, prim)
    sd.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sd.run_cfl(1, ADJ_STEPS)
    sd.synchronize()
    t_plain = time.perf_counter() - t0
    del sd
    # taped forward + backward through the C ABI
    ro = Rollout(mesh, prim)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    traces = ro.forward(1, ADJ_STEPS, ckpt, gauges, obs)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    gp, gz = ro.backward(2.0 * (traces - target))
    t_bwd = time.perf_counter() - t0
    loss = float(np.sum((traces - target) ** 2))
    # the same gradient through torch.autograd
    w0 = torch.tensor(prim[:, 0], dtype=torch.float64, device="cuda", requires_grad=True)
    z = torch.tensor(mesh.geometry[:, 2], dtype=torch.float64, device="cuda", requires_grad=True)
    tr = gauge_rollout(w0, z, mesh, gauges, ADJ_STEPS, obs, ckpt, uv0=prim[:, 1:])
    lt = ((tr - torch.from_numpy(target).cuda()) ** 2).sum()
    lt.backward()
    rel = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    agree = max(rel(w0.grad.cpu().numpy(), gp[:, 0]), rel(z.grad.cpu().numpy(), gz))
    return {"metric": "adjoint/forward time ratio (taped forward + backward) / plain forward",
            "ratio": (t_fwd + t_bwd) / t_plain, "higher_is_better": False, "plain_forward_s": t_plain,
            "taped_forward_s": t_fwd, "backward_s": t_bwd, "cells": mesh.num_cells, "steps": ADJ_STEPS,
            "gauges": 64, "obs_every": obs, "checkpoint_every": ckpt, "loss": loss,
            "grad_norm_w0": float(np.linalg.norm(gp[:, 0])), "grad_norm_z": float(np.linalg.norm(gz)),
            "autograd_vs_c_abi_rel_diff": agree,
            "config": {"workload": "adjoint_250k", "flux": "HLLC+Einfeldt", "scheme": "SSPRK2", "cfl": 0.15}}


BADJ_INSTANCES = int(os.environ.get("SWE_BENCH_BADJ_INSTANCES", "64"))
BADJ_STEPS = int(os.environ.get("SWE_BENCH_BADJ_STEPS", "500"))


def run_batch_adjoint(torch, stream):
    """Batched-adjoint config: 64 seeded instances of 20k-100k cells (the
    ensemble's generator), HLLC + Einfeldt, SSPRK2, per-instance CFL 0.4, 500
    steps, 16 random gauge cells per instance observed every 10th step,
    checkpoint every 25 steps; targets from runs whose bathymetry carries 5%
    seeded Gaussian noise.  Reports (taped forward + backward) / plain batched
    forward, all instances in single launches."""
    from swe_fvm_gb300 import Batch, Fluxes, Wavespeeds, scenarios
    from swe_fvm_gb300.adjoint import BatchRollout
    from swe_fvm_gb300.mesh import Mesh

    t0 = time.time()
    ens = scenarios.adjoint_ensemble(BADJ_INSTANCES)
    t_gen = time.time() - t0
    meshes = [m.contiguous() for m, _ in ens]
    prims = [p for _, p in ens]
    cells = sum(m.num_cells for m in meshes)
    rng = np.random.default_rng(13)
    gauges = [rng.choice(m.num_cells, 16, replace=False) for m in meshes]
    obs, ckpt = 10, 25
    noisy = []
    for m in meshes:
        g = m.geometry.copy()
        g[:, 2] = g[:, 2] * (1.0 + 0.05 * rng.standard_normal(m.num_nodes))
        noisy.append(Mesh(g, m.edge_nodes, m.edge_cells, m.cell_nodes, m.cell_edges, m.cell_neighbours))
    targets = BatchRollout(noisy, prims, cfl=0.4).forward(1, BADJ_STEPS, ckpt, gauges, obs)
    # plain batched forward
    b = Batch(meshes, prims, Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.4)
    b.set_stream(stream.cuda_stream)
    b.run_cfl(1, 2)  # graph capture outside the timed region
    b.synchronize()
    del b
    b = Batch(meshes, prims, Fluxes.HLLC(Wavespeeds.Einfeldt), cfl=0.4)
    b.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run_cfl(1, BADJ_STEPS)
    b.synchronize()
    t_plain = time.perf_counter() - t0
    del b
    br = BatchRollout(meshes, prims, cfl=0.4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    traces = br.forward(1, BADJ_STEPS, ckpt, gauges, obs)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    grads = br.backward([2.0 * (t - tg) for t, tg in zip(traces, targets)])
    t_bwd = time.perf_counter() - t0
    loss = float(sum(np.sum((t - tg) ** 2) for t, tg in zip(traces, targets)))
    return {"metric": "batched adjoint/forward time ratio (taped forward + backward) / plain batched forward",
            "ratio": (t_fwd + t_bwd) / t_plain, "higher_is_better": False, "plain_forward_s": t_plain,
            "taped_forward_s": t_fwd, "backward_s": t_bwd, "instances": len(meshes), "cells": cells,
            "steps": BADJ_STEPS, "gauges_per_instance": 16, "obs_every": obs, "checkpoint_every": ckpt,
            "loss": loss, "grad_norm_z": float(np.sqrt(sum(np.sum(gz ** 2) for _, gz in grads))),
            "config": {"workload": "batched_adjoint_64", "cells_per_instance": "uniform 20k-100k",
                       "flux": "HLLC+Einfeldt", "scheme": "SSPRK2", "cfl": 0.4, "mesh_gen_s": round(t_gen, 1)}}


# DRAM bytes per SSPRK2 step: dram__bytes_read.sum + dram__bytes_write.sum over
# the step's 12 kernels in one ncu capture of the same command line at lattice
# 500 (498,002 cells, tuned order and blocks): 802.8 MB, 1612 B per cell,
# scaled by the cell count to the 999,698-cell mesh (every kernel's bytes grow
# with its cells or edges).
TRAFFIC_PER_STEP = {500: 8.028e8, 708: 1.6115e9}


def run_reference(args):
    """The reference's CPU step on all host threads.  The reference's own
    sources cannot travel to the GPU machine, so this times the C restatement,
    which equals the reference built from its sources bit for bit (Q1/Q20
    edits, tests/test_ref_pin.py), in jacobi loop order on OpenMP threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.oracle import Oracle

    mesh, prim, _ = workload()
    C = mesh.num_cells
    world = int(os.environ.get("WORLD_SIZE", "1"))
    o = Oracle(mesh, prim)
    # every host thread this process may use: the restatement's jacobi-order
    # loops under OpenMP (results equal the single-thread ones bit for bit)
    try:
        threads = len(os.sched_getaffinity(0))
    except AttributeError:
        threads = os.cpu_count() or 1
    o.set_threads(threads)
    o.compute_interface_values()
    o.compute_fluxes()
    for _ in range(args.warmup):
        o.step("SSPRK2", CFL * o.min_len_to_wavespeed())
    budget = 120.0
    done, t = 0, 0.0
    while done < args.steps:
        t0 = time.perf_counter()
        o.step("SSPRK2", CFL * o.min_len_to_wavespeed())
        t += time.perf_counter() - t0
        done += 1
        if t > budget:
            break
    value = C * done / t
    sample = (f"{done} of {args.steps} SSPRK2 steps of the full {C}-cell mesh, {threads} threads ({t:.1f} s); "
              "the C restatement in jacobi loop order (OpenMP), equal bit for bit to the reference's own solver "
              "built from its sources (tests/test_ref_pin.py); the reference's literal loop order runs on one "
              "thread only")
    out = {"impl": "reference", "metric": "cell-updates/s (plain FP64 SSPRK2 step, 1M-triangle unstructured mesh)",
           "value": value, "unit": "cell-updates/s", "n_gpus": world,
           "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * t / done, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(mesh, world),
           "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile", action="store_true", help="only warm-up + K steps (for ncu captures)")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg")
    ap.add_argument("--adjoint-profile", action="store_true", help="only a short taped run and its reverse")
    ap.add_argument("--no-batch-adjoint", action="store_true", help="skip the batched-adjoint leg")
    ap.add_argument("--layouts", action="store_true", help="also time every device order of the mesh")
    ap.add_argument("--ensemble-profile", action="store_true",
                    help="only the batched ensemble: warm-up + K steps (for ncu captures)")
    ap.add_argument("--thacker-profile", action="store_true",
                    help="only the 8192-cell Thacker bowl: warm-up + K steps (for ncu captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
