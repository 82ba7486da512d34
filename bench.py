#!/usr/bin/env python
"""Cell-step throughput of the GB300 path on the headline spheroid workload.

Workload (default): 1,000,000 cells uniform in a ball at density 1 (seed 1),
binned Gabriel finder (cutoff 1.0, c = 0.8), spring force
F = 2*max(0.7-d,0) - 0.5*max(d-0.8,0), Heun dt = 0.05, GlobalComFixer every
step, cell division p = 1e-4 per cell per step (daughter at 0.25 * random unit
vector), capacity 1.05 N.  A step is one Heun step of the whole simulation.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--cells N]

Prints one JSON line (rank 0).  value = cell-steps/s with the state resident
in HBM, each step timed with CUDA events on the simulation's stream and the L2
flushed (256 MiB memset) between steps; e2e = the same metric through the C
ABI with host buffers (pinned upload, per-step agent-count read, download).
Under torchrun every rank runs its own replica (weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-steps/s at 1M cells (Gabriel+Heun)"
UNIT = "cell-steps/s"
# algorithmic bytes per cell of one force pass: read position (float4) + write delta (float4);
# neighbour re-reads are cache reuse and not counted
PASS_BYTES_PER_CELL = 32
# whole Heun + COM step, per cell: bin+reorder 60 + pass 1 32 + pass 2 48 + corrector 64
STEP_BYTES_PER_CELL = 204


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def workload(n_cells: int):
    from tecs_gb300 import workloads as wl

    x = wl.ball(n_cells, 1)
    mn, mx = wl.bounds_for(x, margin=2.0)
    return x, mn, mx


def make_sim(n, mn, mx, device=0):
    import tecs_gb300 as tg

    pf = tg.PairFinderSettings(gabriel_coefficient=0.8, min_bounds=mn, max_bounds=mx)
    cap = int(math.ceil(n * 1.05))
    return tg.Simulation(tg.Settings(agent_count=n, capacity=cap, cutoff_distance=1.0, seed=1, pair_finder_settings=pf),
                         pair_finder="binned_gabriel", integrator="heun", com_fixer="global",
                         force=tg.Spring2R(k_rep=2.0, r_rep=0.7, k_adh=0.5, r_adh=0.8),
                         division=tg.Division(probability=1e-4, offset=0.25), device=device)


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [t.strip() for t in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def traffic_per_pass():
    """DRAM bytes per k_pass launch from the committed ncu capture, scaled to 1M cells."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return d.get("k_pass_store_bytes_per_cell")
    except Exception:
        return None


def cpu_baseline(n_cells, steps, threads, budget_s=20.0):
    """The oracle (C restatement, OpenMP) on a bounded sample of the same workload."""
    import oracle
    from tecs_gb300 import workloads as wl

    x, mn, mx = workload(n_cells)
    cap = int(math.ceil(n_cells * 1.05))
    o = oracle.Oracle(finder=oracle.BINNED_GABRIEL, integrator=oracle.HEUN, com_fix=True, min_bounds=mn,
                      max_bounds=mx, capacity=cap, division_probability=1e-4, division_offset=0.25, seed=1)
    o.set_state(x)
    t0 = time.perf_counter()
    o.step(0.05, 1, threads)  # warm-up
    first = time.perf_counter() - t0
    k = max(1, min(steps, int(budget_s / max(first, 1e-3))))
    cs = 0
    t0 = time.perf_counter()
    for _ in range(k):
        n = o.count
        o.step(0.05, 1, threads)
        cs += n
    dt = time.perf_counter() - t0
    return cs / dt, k, dt


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n = args.cells
    # the reference's algorithm on the host cores: the oracle's C restatement with OpenMP
    x, mn, mx = workload(n)
    import oracle

    cap = int(math.ceil(n * 1.05))
    o = oracle.Oracle(finder=oracle.BINNED_GABRIEL, integrator=oracle.HEUN, com_fix=True, min_bounds=mn,
                      max_bounds=mx, capacity=cap, division_probability=1e-4, division_offset=0.25, seed=1)
    o.set_state(x)
    for _ in range(args.warmup):
        o.step(0.05, 1, threads)
    # bounded sample: at most --steps steps and about 60 s
    cs, k = 0, 0
    t0 = time.perf_counter()
    while k < args.steps and (time.perf_counter() - t0) < 60.0:
        cs += o.count
        o.step(0.05, 1, threads)
        k += 1
    dt = time.perf_counter() - t0
    v = cs / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(k, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"spheroid {n} cells, binned Gabriel, spring, Heun dt 0.05, COM, division 1e-4",
                   "cells": n, "l2": "n/a (host)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{k} Heun steps of the {n}-cell spheroid after {args.warmup} warm-up"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import torch

    import tecs_gb300 as tg

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    n = args.cells
    x, mn, mx = workload(n)
    sim = make_sim(n, mn, mx, device=local)
    stream = torch.cuda.ExternalStream(sim.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    xd = torch.from_numpy(x).to("cuda")
    torch.cuda.synchronize()
    sim.set_state_device(xd.data_ptr(), None, n)
    sim.set_profiling(True)

    for _ in range(args.warmup):
        sim.take_step(0.05)
    sim.synchronize()

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    step_ms, kern = [], {}
    cell_steps = 0
    with Clocks(local) as clocks:
        for _ in range(args.steps):
            nb = sim.get_agent_count()
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            sim.take_step(0.05)
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            step_ms.append(e0.elapsed_time(e1))
            for name, ms in sim.last_step_profile():
                kern.setdefault(name, []).append(ms)
            cell_steps += nb
    torch.cuda.synchronize()
    total_s = sum(step_ms) / 1e3
    if world > 1:
        t = torch.tensor([total_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
        c = torch.tensor([cell_steps], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(c)
        cell_steps_all = float(c.item())
    else:
        cell_steps_all = float(cell_steps)
    torch.cuda.synchronize()
    value = cell_steps_all / total_s
    kpl = sim.kernels_per_step()

    # end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        L = tg.load()
        cap = sim.desc.capacity
        hx = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
        hx.numpy()[:] = x
        hout = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True)
        nn = ctypes.c_uint()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tg._check(L.tecs_sim_upload(sim._h, ctypes.c_void_p(hx.data_ptr()), None, n))
        cs = 0
        for _ in range(args.steps):
            tg._check(L.tecs_sim_count(sim._h, ctypes.byref(nn)))
            cs += nn.value
            tg._check(L.tecs_sim_step(sim._h, 0.05, 1))
        tg._check(L.tecs_sim_download(sim._h, ctypes.c_void_p(hout.data_ptr()), None, ctypes.byref(nn)))
        t1 = time.perf_counter()
        e2e = {"value": cs / (t1 - t0), "unit": UNIT,
               "h2d_bytes_per_step": int(n * 12 / args.steps),
               "d2h_bytes_per_step": int(4 + nn.value * 12 / args.steps),
               "note": "pinned upload of the initial state and final download amortised over the steps; "
                       "agent count read back every step"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    hbm, peak_kind = peaks()
    passes = [ms for name, v in kern.items() if name.startswith("k_pass") for ms in v]
    n_avg = cell_steps / max(args.steps, 1)
    pass_ms = statistics.mean(passes) if passes else float("nan")
    achieved = PASS_BYTES_PER_CELL * n_avg / (pass_ms / 1e3) / 1e9
    tpc = traffic_per_pass()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": (tpc * n_avg if tpc else None), "kernel": "k_pass (Gabriel + spring force pass)",
                "bytes_per_cell": PASS_BYTES_PER_CELL, "peak_kind": f"{peak_kind} hbm_gbs",
                "avg_launch_ms": pass_ms}
    step_achieved = STEP_BYTES_PER_CELL * n_avg / (statistics.mean(step_ms) / 1e3) / 1e9
    kernel_table = {k: {"launches": len(v), "mean_ms": statistics.mean(v), "share": sum(v) / max(sum(step_ms), 1e-9)}
                    for k, v in kern.items()}
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        threads = os.cpu_count() or 1
        v, k, dt = cpu_baseline(n, 64, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{k} Heun steps of the {n}-cell spheroid after 1 warm-up ({dt:.1f} s, OpenMP)"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(step_ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"spheroid {n} cells, binned Gabriel, spring, Heun dt 0.05, COM, division 1e-4",
                   "cells": n, "capacity": sim.desc.capacity, "bins": None,
                   "l2": "flushed between timed steps (256 MiB memset)", "parallelism": f"replicas x{world}"},
        "roofline": roofline,
        "step_roofline": {"bytes_per_cell": STEP_BYTES_PER_CELL, "achieved": step_achieved, "frac": step_achieved / hbm},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": kpl * args.steps,
        "kernels": kernel_table,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_ensemble(args):
    """Batched form vs the plain drop-in run sequentially, on the 256-simulation ensemble."""
    import torch

    from tecs_gb300 import batched

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    members = batched.ensemble(args.sims, 2)
    cells = sum(len(m.x) for m in members)
    scales, timings = ({}, {}) if args.no_tune else batched.autotune(members)
    eng, _ = batched.build_engine(members, scales, device=local)
    with Clocks(local) as clocks:
        t_b = batched.time_engine_steps(eng, args.steps, warmup=args.warmup)
    kpl = eng.kernels_per_step()
    eng.close()
    t_p = batched.run_plain_steps_only(members, args.steps)
    v_b = cells * args.steps / t_b
    v_p = cells * args.steps / t_p
    line = {
        "metric": "cell-steps/s, 256-simulation ensemble (batched)", "value": v_b, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_b / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{len(members)} simulations, cells log-uniform in [500, 200000] (seed 2), "
                               "density-1 balls, 50% Gabriel / 50% binned all-pairs, Heun dt 0.05",
                   "cells": cells, "l2": "state larger than L2", "bin_size_scale": scales,
                   "autotune_seconds_per_4_steps": timings},
        "plain_sequential": {"value": v_p, "ms_per_step_all_sims": 1e3 * t_p / args.steps},
        "speedup_vs_plain": v_b / v_p,
        "gpu_launches": kpl * args.steps,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cells", type=int, default=1_000_000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="spheroid", choices=["spheroid", "ensemble", "served"])
    ap.add_argument("--sims", type=int, default=256)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--requests", type=int, default=200, help="served workload: number of requests")
    ap.add_argument("--time-scale", type=float, default=1.0, help="served workload: arrival-time compression")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "served":
        from tecs_gb300 import served
        return served.bench_main(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
