#!/usr/bin/env python
"""Throughput of the GB300 Euler solver: cell-stage updates per second.

A "step" is one solver iteration (all RK stages of the explicit scheme) over
the whole mesh; one cell-stage update is one RK stage applied to one cell, so
value = ncell * stages * steps / time.

Default workload: the large-mesh configuration -- NACA 0012 O-grid 2048 x 1024
(4,194,304 triangles, seeded diagonals and 5% jitter), Morton-ordered cells,
M 0.78, alpha 2.0 deg, FP32 stencil with FP64 geometry and residual norm,
residual smoothing on (2 sweeps), the reference's 4-stage RK.  Its working set
(~1 GB) is far larger than the 129 MB L2, so no L2 flush is needed between
steps.

Arms:
  --impl gb300      (default) the CUDA path through the C ABI
  --impl reference  the CPU path of the reference scheme (the oracle port of
                    its GPU loop, OpenMP on all host cores) on the same
                    workload, one iteration per step

N > 1 (torchrun): replicas only -- the reference path has no domain
decomposition; each rank solves its own copy, no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: mesh size, flow conditions and description; the arithmetic type of
    # a run (FP32 stencil with FP64 geometry / norms, or FP64 throughout) is
    # the line's "dtype", not part of the workload
    "large": dict(ni=2048, nj=1024, ma=0.78, alpha=2.0, cfl=2.0,
                  desc="NACA0012 O-grid 2048x1024 (4194304 tri), Morton, M0.78 a2.0, CFL 2, "
                       "IRS 2 sweeps eps 0.8, 4-stage RK"),
    "medium": dict(ni=1024, nj=512, ma=0.78, alpha=2.0, cfl=2.0,
                   desc="NACA0012 O-grid 1024x512 (1048576 tri), Morton, M0.78 a2.0, CFL 2, "
                        "IRS 2 sweeps eps 0.8, 4-stage RK"),
    "transonic": dict(ni=512, nj=128, ma=0.80, alpha=1.25, cfl=2.0,
                      desc="NACA0012 O-grid 512x128 (131072 tri), Morton, M0.80 a1.25, CFL 2, "
                           "IRS 2 sweeps eps 0.8, 4-stage RK"),
}

def l2_note(ncell: int) -> str:
    """How the timed iterations avoid a warm L2: the large meshes' working set
    (~270 B per cell in FP32) is several times the 129 MB L2."""
    if ncell * 270 > 4 * 129e6:
        return f"inputs larger than L2 (working set ~{ncell * 270 / 1e9:.1f} GB), no flush"
    return "working set fits in L2 (not a roofline case), no flush"


def cpu_model() -> str:
    """The host CPU's model name (lscpu), for the CPU baseline records."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        fields = {k.strip(): v.strip() for k, _, v in (line.partition(":") for line in out.splitlines())}
        name = " ".join(v for v in (fields.get("Vendor ID"), fields.get("Model name")) if v and v != "-")
        if name:
            return name
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.processor() or platform.machine()

PASS_NAMES = ["faces", "flux", "smooth", "update", "resid"]


def bytes_per_cell(prec_bytes: int) -> dict:
    """Algorithmic (compulsory) bytes per cell of each pass, from the arrays it
    touches: every element read or written once per launch, neighbour gathers
    perfectly reused.  T = stencil precision, int4 topology 16 B."""
    T = prec_bytes
    topo = 16
    W, S2x3, R2x3, A, FS, dt, V4 = 4 * T, 6 * T, 6 * T, T, 12 * T, T, 4 * T
    Af = A
    if T == 4:
        R2x3, Af = 0, 0  # the FP32 pass A derives face offsets and area from S
    return {
        "faces": W + topo + S2x3 + R2x3 + Af + FS + dt,  # reads W,topo,S,(R,area) -> FS, dt
        "flux": topo + S2x3 + FS + V4,                   # reads topo,S,FS -> res
        "smooth": topo + V4 + V4 + V4,                   # reads topo,src,res -> dst
        "update": topo + V4 + V4 + dt + A + V4 + V4,     # topo,src,res,dt,area,W0 -> W
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index
        out = os.environ.get("E2D_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out, f"e2d_clocks_gpu{gpu_index}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = max(smax, float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def measured_peak_bf16() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def max_over_ranks(t: float, dist, device: str) -> float:
    """The slowest rank's time (the job's time); t itself without a process group."""
    if dist is None:
        return t
    import torch
    v = torch.tensor([t], dtype=torch.float64, device=device)
    dist.all_reduce(v, op=dist.ReduceOp.MAX)
    return float(v.item())


def replica_rate(world: int, ncell: int, stages: int, steps: int, t_max: float) -> float:
    """Whole-job cell-stage updates/s of `world` replicas that each ran `steps`
    iterations of an ncell-cell mesh, timed by the slowest one."""
    return world * ncell * stages * steps / t_max


ORDERINGS = {"morton": ("E2D_ORDER_MORTON", "Morton"), "rcm": ("E2D_ORDER_RCM", "RCM"),
             "file": ("E2D_ORDER_FILE", "file order")}


def make_params(e2d, wl, precision, block=0, ordering="morton"):
    return e2d.default_params(ma=wl["ma"], alpha_deg=wl["alpha"], cfl=wl["cfl"], precision=precision,
                              ordering=getattr(e2d, ORDERINGS[ordering][0]), maxstep=1000000, block_size=block)


def workload_desc(wl, ordering="morton") -> str:
    return wl["desc"].replace("Morton", ORDERINGS[ordering][1])


def cpu_port_rate(wl, steps_wanted: float, threads: int | None = None):
    """Oracle port of the reference loop on the host cores, on the oracle's
    own statement of the same mesh: returns (cell-stage/s, iterations run,
    seconds, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    x, y, tri = pyoracle.ogrid(wl["ni"], wl["nj"], seed=1)
    p = pyoracle.params(ma=wl["ma"], alpha_deg=wl["alpha"], cfl=wl["cfl"])
    case = pyoracle.Case(x, y, tri, p)
    if threads:
        pyoracle.set_threads(threads)
    th = pyoracle.threads()
    n = max(1, int(steps_wanted))
    t0 = time.perf_counter()
    k = len(case.run(n))
    dt = time.perf_counter() - t0
    return case.ncell * p.rk_stages * k / dt, k, dt, th


def run_reference(args, rank: int, world: int):
    """--impl reference: the reference scheme's CPU path on the host cores.
    This arm loads only the oracle (its mesh comes from the oracle's statement
    of the O-grid generator, equal bit for bit to the library's), never the
    product library."""
    if rank != 0:
        return
    wl = WORKLOADS[args.workload]
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    x, y, tri = pyoracle.ogrid(wl["ni"], wl["nj"], seed=1)
    p = pyoracle.params(ma=wl["ma"], alpha_deg=wl["alpha"], cfl=wl["cfl"])
    case = pyoracle.Case(x, y, tri, p)
    th = pyoracle.threads()
    # warm-up, timing the last warm-up iteration to size the timed sample so
    # the run stays within about a minute of host time
    case.run(max(0, args.warmup - 1))
    t0 = time.perf_counter()
    case.run(1)
    t_it = time.perf_counter() - t0
    k_want = max(1, min(args.steps, int(60.0 / max(t_it, 1e-6))))
    t0 = time.perf_counter()
    k = len(case.run(k_want))
    dt = time.perf_counter() - t0
    rate = case.ncell * p.rk_stages * k / dt
    line = {
        "impl": "reference", "metric": "cell-stage updates/s", "value": rate, "unit": "cell-stage/s",
        "n_gpus": world, "steps": k, "warmup": args.warmup, "ms_per_step": dt / k * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded NACA0012 O-grid)",
        "config": {"workload": workload_desc(wl, args.ordering), "cells": case.ncell, "stages": p.rk_stages,
                   "parallelism": f"replicas{world}", "l2": l2_note(case.ncell)},
        "cpu_baseline": {"value": rate, "unit": "cell-stage/s", "cores": th, "cpu_model": cpu_model(),
                         "kind": "port",
                         "sample": f"{k} of the {args.steps} requested iterations (capped at ~60 s of host "
                                   f"time) of the full {case.ncell}-cell workload, FP64 (the reference's "
                                   f"precision), cells in file order, on {th} threads"},
        "e2e": {"value": rate, "unit": "cell-stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, rank: int, world: int):
    import numpy as np
    import torch
    import gpueularsolver2d_gb300 as e2d

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl = WORKLOADS[args.workload]
    prec = e2d.E2D_FP64 if args.fp64 else e2d.E2D_FP32
    t_setup0 = time.perf_counter()
    mesh = e2d.Mesh.ogrid(wl["ni"], wl["nj"], seed=1)
    t_setup1 = time.perf_counter()
    params = make_params(e2d, wl, prec, args.block, args.ordering)
    solver = e2d.Solver(mesh, params)  # set-up: geometry, edges, tags, cell order, layout, upload
    torch.cuda.synchronize()
    setup = {"mesh_generation_s": t_setup1 - t_setup0, "solver_create_s": time.perf_counter() - t_setup1}
    ncell, stages = solver.ncell, params.rk_stages
    launches = solver.launches_per_iteration()

    def barrier():
        if dist is not None:
            dist.barrier()

    solver.step(args.warmup)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    solver.step(args.steps)          # CUDA events on the solver's stream bracket the K steps
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    dev_ms = solver.last_device_ms()
    barrier()
    clocks = sampler.stop()
    t_local = dev_ms / 1e3
    t_max = max_over_ranks(t_local, dist, "cuda")
    value = replica_rate(world, ncell, stages, args.steps, t_max)

    # per-pass device time inside the same iteration sequence (events around every launch)
    prof_iters = 3
    ms, nl = solver.profile_passes(prof_iters)
    tbytes = 8 if prec == e2d.E2D_FP64 else 4
    bpc = bytes_per_cell(tbytes)
    per_pass = {}
    for k, name in enumerate(PASS_NAMES):
        if nl[k] == 0:
            continue
        avg = ms[k] / nl[k]
        entry = {"launches": int(nl[k]), "avg_ms": avg, "share": ms[k] / ms.sum()}
        if name in bpc:
            entry["algo_bytes_per_launch"] = bpc[name] * ncell
            entry["achieved_gbs"] = bpc[name] * ncell / (avg / 1e3) / 1e9
        per_pass[name] = entry
    dom = max((n for n in per_pass if n in bpc), key=lambda n: per_pass[n]["avg_ms"] * per_pass[n]["launches"])
    peak, peak_kind = measured_peak_hbm()
    achieved = per_pass[dom]["achieved_gbs"]
    stage_bytes = sum(bpc[n] * (args_sweeps_count(params) if n == "smooth" else 1) for n in bpc)
    roofline = {"bound": "hbm", "kernel": f"k_{dom}", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)",
                "traffic": traffic_from_profiles(dom, ncell),
                "algo_bytes_per_cell_stage": stage_bytes,
                "whole_step_frac": stage_bytes * ncell * stages * args.steps / t_local / 1e9 / peak}

    # end to end through the C ABI with host buffers: every step uploads the
    # state from pinned host memory, iterates once and reads the state back
    pin_in = torch.empty((ncell, 4), dtype=torch.float64, pin_memory=True).numpy()
    pin_out = torch.empty((ncell, 4), dtype=torch.float64, pin_memory=True).numpy()
    pin_in[:] = solver.state()
    e2e_steps = max(3, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.set_state(pin_in)
        solver.step(1)
        solver.state_into(pin_out)
    torch.cuda.synchronize()
    e2e_t = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    e2e_rate = replica_rate(world, ncell, stages, e2e_steps, e2e_t)

    # FP32 stencil against an FP64 run of the same code on the same workload:
    # after one iteration (the stencil's own rounding) and after 20 (where the
    # start-up transient has begun to amplify rounding differences)
    fp_err = None
    if rank == 0 and prec == e2d.E2D_FP32:
        a32 = e2d.Solver(mesh, make_params(e2d, wl, e2d.E2D_FP32, ordering=args.ordering))
        a64 = e2d.Solver(mesh, make_params(e2d, wl, e2d.E2D_FP64, ordering=args.ordering))
        fp_err = {}
        for n_err, key in ((1, "after_1_iteration"), (19, "after_20_iterations")):
            a32.step(n_err)
            a64.step(n_err)
            w32, w64 = a32.state(), a64.state()
            h32, h64 = a32.history(), a64.history()
            fp_err[key] = {"max_rel_linf": float(np.max(np.abs(w32 - w64)) / np.max(np.abs(w64))),
                           "median_rel": float(np.median(np.abs(w32 - w64) / np.abs(w64).max(axis=0))),
                           "resid_max_rel": float(np.max(np.abs(h32 - h64) / h64))}
            try:
                fp_err[key]["integrals"] = integral_errors(a32.integrals(), a64.integrals())
            except Exception as exc:  # an auxiliary report: keep the bench line, say why it is missing
                fp_err[key]["integrals"] = {"error": str(exc)}
        a32.close()
        a64.close()

    # the same workload with the FP64 stencil (the reference's precision):
    # device time of a few iterations and the per-pass split
    fp64 = None
    if rank == 0 and prec == e2d.E2D_FP32 and not args.no_fp64:
        solver = None
        torch.cuda.synchronize()
        s64 = e2d.Solver(mesh, make_params(e2d, wl, e2d.E2D_FP64, ordering=args.ordering))
        k64 = max(1, min(args.fp64_steps, args.steps))
        s64.step(2)
        s64.step(k64)
        t64 = s64.last_device_ms() / 1e3
        ms64, nl64 = s64.profile_passes(1)
        fp64 = {"value": ncell * stages * k64 / t64, "unit": "cell-stage/s", "steps": k64,
                "ms_per_step": t64 / k64 * 1e3, "dtype": "f64",
                "passes_ms_per_step": {name: float(ms64[j]) for j, name in enumerate(PASS_NAMES) if nl64[j]},
                "launches_per_step": {name: int(nl64[j]) for j, name in enumerate(PASS_NAMES) if nl64[j]}}
        s64.close()
    # the two other forms of the benchmark spec on the same box, as sub-records:
    # the 64-case batched sweep and the warm-start network's training step
    extras = {}
    if rank == 0 and not args.no_extras:
        solver = None
        torch.cuda.synchronize()
        for name, fn in (("batched_sweep", lambda: batch64_record(50, 5)),
                         ("mlp_training", lambda: mlp_record(args.mlp_layers, 50, 5))):
            try:
                extras[name] = fn()
            except Exception as exc:  # an auxiliary record: keep the bench line, say why it is missing
                extras[name] = {"error": str(exc)}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        solver = None
        torch.cuda.synchronize()
        rate, k, dt, th = cpu_port_rate(wl, 2)
        rate1, k1, dt1, _ = cpu_port_rate(wl, 1, threads=1)
        cpu = {"value": rate, "unit": "cell-stage/s", "cores": th, "cpu_model": cpu_model(), "kind": "port",
               "sample": f"{k} iterations of the full {ncell}-cell workload, FP64, on {th} threads ({dt:.1f} s)",
               "single_thread_value": rate1,
               "single_thread_sample": f"{k1} iteration on 1 thread ({dt1:.1f} s)"}
    if rank == 0:
        line = {
            "metric": "cell-stage updates/s", "value": value, "unit": "cell-stage/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == e2d.E2D_FP64 else "f32",
            "data": "synthetic (seeded NACA0012 O-grid)",
            "config": {"workload": workload_desc(wl, args.ordering), "cells": ncell, "stages": stages,
                       "parallelism": f"replicas{world}", "l2": l2_note(ncell)},
            "wall_ms_per_step": wall / args.steps * 1e3,
            "roofline": roofline, "passes": per_pass, "fp32_error_vs_fp64": fp_err, "fp64": fp64, "setup": setup,
            **extras,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_rate, "unit": "cell-stage/s", "steps": e2e_steps,
                    "h2d_bytes_per_step": int(pin_in.nbytes), "d2h_bytes_per_step": int(pin_out.nbytes)},
            "gpu_launches": launches * args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def batch64_record(steps: int, warmup: int) -> dict:
    """Batched sweep: 64 cases on O-grids of sizes drawn from {64..512}x{16..128}
    (seed 2), Mach U[0.3, 0.85], alpha U[-2, 4] deg, FP32, one launch per pass
    over all cases with the cell order and launch shape picked by the
    autotuner, against the same 64 cases solved one after the other by the
    single-case solver (device time of `steps` iterations each)."""
    import numpy as np
    import gpueularsolver2d_gb300 as e2d
    rng = np.random.default_rng(2)
    ni = rng.choice([64, 128, 256, 512], 64)
    nj = rng.choice([16, 32, 64, 128], 64)
    mach = rng.uniform(0.3, 0.85, 64)
    alpha = rng.uniform(-2.0, 4.0, 64)
    meshes = [e2d.Mesh.ogrid(int(a), int(b), seed=10 + k) for k, (a, b) in enumerate(zip(ni, nj))]
    params = [e2d.default_params(ma=float(m), alpha_deg=float(a), cfl=2.0, precision=e2d.E2D_FP32,
                                 ordering=e2d.E2D_ORDER_MORTON, maxstep=steps + warmup + 64)
              for m, a in zip(mach, alpha)]
    cells = sum(2 * int(a) * int(b) for a, b in zip(ni, nj))
    t0 = time.perf_counter()
    b = e2d.Batch.tuned(meshes, params, None, iters=16)
    t_tune = time.perf_counter() - t0
    block, grid = b.launch()
    order_name = {e2d.E2D_ORDER_MORTON: "Morton", e2d.E2D_ORDER_RCM: "RCM", e2d.E2D_ORDER_FILE: "file"}[b.ordering]
    b.step(warmup)
    b.step(steps)
    t_batch = b.last_device_ms() / 1e3
    stages = params[0].rk_stages
    agg = cells * stages * steps / t_batch
    launches = b.launches_per_iteration()
    b.close()
    t_seq = 0.0
    for m, p in zip(meshes, params):
        s = e2d.Solver(m, p)
        s.step(warmup)
        s.step(steps)
        t_seq += s.last_device_ms() / 1e3
        s.close()
    seq = cells * stages * steps / t_seq
    return {"metric": "cell-stage updates/s (64-case batched sweep)", "value": agg, "unit": "cell-stage/s",
            "steps": steps, "warmup": warmup, "ms_per_step": t_batch / steps * 1e3, "dtype": "f32",
            "config": {"workload": "64 cases, O-grids {64..512}x{16..128} (seed 2), M U[0.3,0.85], a U[-2,4]",
                       "cells": cells, "stages": stages, "autotuned_block": block, "autotuned_grid": grid,
                       "autotuned_ordering": order_name, "autotune_seconds": t_tune},
            "sequential_value": seq, "speedup_vs_sequential": agg / seq, "gpu_launches": launches * steps}


def run_batch64(args):
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rec = batch64_record(args.steps, args.warmup)
    line = {"metric": rec.pop("metric"), "value": rec.pop("value"), "unit": rec.pop("unit"), "n_gpus": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded NACA0012 O-grids)", **rec}
    print(json.dumps(line), flush=True)


def mlp_record(layers: int, steps: int, warmup: int) -> dict:
    """Training steps of the warm-start MLP (22 features padded to 32 -> L x
    256 GELU -> 4, batch 65536, BF16 tensor-core GEMMs with FP32 accumulate):
    gather, forward, loss, backward and Adam of one step are one CUDA graph.
    FLOPs per step: the tensor-core GEMMs, 2 B (32 * 256 + (L - 1) * 256^2)
    each for the forward pass and the weight gradients and 2 B (L - 1) * 256^2
    for the data gradients (the first layer needs none); the 256 -> 4 output
    layer runs on the CUDA cores and is not counted."""
    import numpy as np
    import torch
    import gpueularsolver2d_gb300 as e2d
    L, B = layers, 65536
    # the warp-specialised hidden-layer kernels or an error, never the per-tile fallback
    os.environ.setdefault("E2D_MLP_WS", "1")
    net = e2d.MLP(nhidden=L, batch=B, seed=3)
    rng = np.random.default_rng(0)
    n = 32768 * 64
    x = np.zeros((n, 32), np.float32)
    x[:, :22] = rng.uniform(-1, 1, (n, 22))
    t = rng.normal(size=(n, 4)).astype(np.float32)
    net.set_data(x, t)
    net.train(warmup, record_loss=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net.train(steps, record_loss=False)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    net.close()
    flops = 2 * B * (2 * (32 * 256 + (L - 1) * 256 * 256) + (L - 1) * 256 * 256)
    peak, kind = measured_peak_bf16()
    tf = flops / dt / 1e12
    return {"metric": "MLP training steps/s (warm-start network, batch 65536)", "value": 1.0 / dt, "unit": "steps/s",
            "steps": steps, "warmup": warmup, "ms_per_step": dt * 1e3, "dtype": "bf16",
            "config": {"workload": f"MLP 32 -> {L} x 256 GELU -> 4, batch {B}, Adam"},
            "roofline": {"bound": "tensor", "achieved": tf, "peak": peak, "unit": "TFLOP/s", "frac": tf / peak,
                         "peak_source": f"{kind} bf16_tflops (MEASURED_PEAKS.json)", "traffic": None},
            # per step: step counter, gather, L forward GEMMs, the output layer,
            # L weight gradients, L - 1 data gradients, L + 1 Adam launches
            "gpu_launches": (4 * L + 3) * steps}


def run_mlp(args):
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rec = mlp_record(args.mlp_layers, args.steps, args.warmup)
    line = {"metric": rec.pop("metric"), "value": rec.pop("value"), "unit": rec.pop("unit"), "n_gpus": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (uniform features, normal targets)", **rec}
    print(json.dumps(line), flush=True)


def integral_errors(i32: dict, i64: dict) -> dict:
    """FP64 integrals (e2d_integrals) of the FP32 run against those of the FP64
    run: both values and their absolute difference."""
    return {k: {"fp32": i32[k], "fp64": i64[k], "abs_err": abs(i32[k] - i64[k])}
            for k in ("cl", "cd", "mass", "mass_flux_far", "mass_flux_wall")}


def args_sweeps_count(params) -> int:
    return max(0, params.irs_sweeps - 1)


def traffic_from_profiles(kernel: str, ncell: int):
    """DRAM bytes per launch from the committed ncu summary, scaled to ncell."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        e = t[f"k_{kernel}"]
        return e["dram_bytes_per_cell"] * ncell
    except (OSError, KeyError, ValueError):
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batch64", "mlp"], default="large")
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--block", type=int, default=0, help="threads per CTA (0: library default)")
    ap.add_argument("--ordering", choices=sorted(ORDERINGS), default="morton", help="cell order in device memory")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64-stencil record of the same workload")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched-sweep and MLP-training sub-records of the default line")
    ap.add_argument("--fp64-steps", type=int, default=10, help="timed iterations of the FP64-stencil record")
    ap.add_argument("--mlp-layers", type=int, default=8, help="hidden layers of the MLP workload")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.workload == "mlp":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned warm start"}))
        elif rank == 0:
            run_mlp(args)
    elif args.workload == "batch64":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference solves one case per run; "
                              "the batched sweep has no reference arm"}))
        elif rank == 0:
            run_batch64(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)


if __name__ == "__main__":
    main()
