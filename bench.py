#!/usr/bin/env python
"""Cell-step throughput of the GB300 path.

Workloads (--workload):
  spheroid (default, the headline): 1,000,000 cells uniform in a ball at
      density 1 (seed 1), binned Gabriel finder (cutoff 1.0, c = 0.8), spring
      force F = 2*max(0.7-d,0) - 0.5*max(d-0.8,0), Heun dt = 0.05,
      GlobalComFixer every step, cell division p = 1e-4 per cell per step
      (daughter at 0.25 * random unit vector), capacity 1.05 N (grown when a
      run's expected divisions need more).
  sheet: 100,000 cells on a sphere of radius sqrt(N/4pi)*0.8 (jitter 0.02),
      outward polarity + N(0, 0.1), binned Gabriel, spring + 0.2 (bending +
      alignment), Heun dt = 0.05.
  small: 1,000 cells in a ball of radius 5 (seed 0), binned all-pairs, spring,
      Euler dt = 0.1.
  delaunay, delaunay3d: 100,000 cells uniform in a 2-D disk or a 3-D ball at
      density 1, the Delaunay finder of any capacity (cutoff 1.0), spring,
      Heun dt = 0.05 (no CPU leg: the reference's naive Delaunay finder does
      O(N^3) work per cell).
  ensemble: 256 simulations in one engine vs the plain path one after another.
  served: the continuous-batching request loop (tecs_gb300.served).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload W] [--cells N]

Prints one JSON line (rank 0).  value = cell-steps/s with the state resident
in HBM: each timed step is --chunk simulation steps (default 10, so the
default 20 timed steps run the spheroid's 200), timed with CUDA events on the
simulation's stream, the L2 flushed (256 MiB memset) before each; the default
spheroid line also carries the 256-simulation ensemble, batched against the
plain path one simulation after another.  e2e = the same metric through the C
ABI with host buffers (every step: pinned upload of the state, the step, and
the download of the new state).  --impl reference times the reference's
algorithm (the oracle's C restatement, OpenMP) on the host cores.  Under
torchrun every rank runs its own replica (weak scaling, no collective).
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

# Algorithmic bytes per cell of one force-pass launch, by pass kind: each
# cell's own state read once and its outputs written once (float4 position /
# delta, float2 polarity); neighbour re-reads are cache reuse and not counted.
PASS_BYTES = {
    "k_pass_store": (32, 16),   # read x, write delta             (+ read p, write dp)
    "k_pass_euler": (32, 16),   # read x, write x'                (+ p, p')
    "k_pass_heun1": (48, 24),   # read x, write d1, x~            (+ p, dp1, p~)
    "k_pass_heun2": (64, 32),   # read x~, x, d1, write x'        (+ p~, p, dp1, p')
    "k_step_small": (32, 16),   # the one-launch Euler step: read x, write x' (+ p, p')
}


def _ball_workload(n):
    from tecs_gb300 import workloads as wl

    x = wl.ball(n, 1)
    mn, mx = wl.bounds_for(x, margin=2.0)
    return x, None, mn, mx


def _sheet_workload(n):
    from tecs_gb300 import workloads as wl

    x = wl.sheet(n, 1)
    p = wl.outward_polarity(x, 1)
    mn, mx = wl.bounds_for(x, margin=2.0)
    return x, p, mn, mx


def _disk_workload(n):
    from tecs_gb300 import workloads as wl

    x = wl.disk(n, 1)
    mn, mx = wl.bounds_for(x, margin=2.0)
    return x, None, mn, mx


def _small_workload(n):
    from tecs_gb300 import workloads as wl

    x = wl.ball(n, 0, radius=5.0)
    return x, None, (-6.0,) * 3, (6.0,) * 3


# The configurations this benchmark runs.  spheroid is the headline (the
# metric's 1M-cell Gabriel + Heun step); sheet and small are the epithelial
# sheet with polarity and the small plain configuration.
WORKLOADS = {
    "spheroid": dict(
        metric=METRIC, cells=1_000_000, make=_ball_workload, finder="binned_gabriel", integrator="heun", com=True,
        division=1e-4, polarity=False, dt=0.05, capacity=1.05,
        desc="spheroid {n} cells, binned Gabriel, spring, Heun dt 0.05, COM, division 1e-4",
        step_bytes=204),  # bin+reorder 60, pass 1 32, pass 2 48, corrector 64
    "sheet": dict(
        metric="cell-steps/s, 100k-cell epithelial sheet (Gabriel + polarity, Heun)", cells=100_000,
        make=_sheet_workload, finder="binned_gabriel", integrator="heun", com=False, division=0.0, polarity=True,
        dt=0.05, capacity=1.0,
        desc="sheet {n} cells on a sphere (R = sqrt(N/4pi)*0.8, jitter 0.02), binned Gabriel, spring + "
             "0.2 (bending + alignment), Heun dt 0.05",
        step_bytes=212),  # Heun without COM 156 + polarity 56
    "small": dict(
        metric="cell-steps/s, 1k-cell plain small (binned all-pairs, Euler)", cells=1000, make=_small_workload,
        finder="binned_all_pairs", integrator="euler", com=False, division=0.0, polarity=False, dt=0.1,
        capacity=1.0, desc="ball {n} cells radius 5 (seed 0), binned all-pairs, spring, Euler dt 0.1",
        step_bytes=92),
    # the Delaunay finder of any capacity; the reference's naive finder does
    # O(N^3) work per cell, so no CPU leg runs at this size
    "delaunay": dict(
        metric="cell-steps/s, 100k-cell 2-D disk (Delaunay finder, spring, Heun)", cells=100_000,
        make=_disk_workload, finder="delaunay", integrator="heun", com=False, division=0.0, polarity=False,
        dt=0.05, capacity=1.0, dims=2, cpu=False,
        desc="disk {n} cells (density 1, seed 1), Delaunay finder, spring, Heun dt 0.05", step_bytes=156),
    "delaunay3d": dict(
        metric="cell-steps/s, 100k-cell 3-D ball (Delaunay finder, spring, Heun)", cells=100_000,
        make=_ball_workload, finder="delaunay", integrator="heun", com=False, division=0.0, polarity=False,
        dt=0.05, capacity=1.0, dims=3, cpu=False,
        desc="ball {n} cells (density 1, seed 1), Delaunay finder, spring, Heun dt 0.05", step_bytes=156),
}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def capacity_for(w, n, steps=0):
    """The workload's capacity (>= its stated fraction of n), grown to hold the
    expected divisions over `steps` steps with 2 % to spare."""
    grow = (1.0 + w["division"]) ** steps * 1.02 if w["division"] > 0 else 1.0
    return int(math.ceil(n * max(w["capacity"], grow)))


def make_sim(w, n, mn, mx, device=0, steps=0):
    import tecs_gb300 as tg

    pf = tg.PairFinderSettings(gabriel_coefficient=0.8, min_bounds=mn, max_bounds=mx)
    cap = capacity_for(w, n, steps)
    force = tg.PolaritySpring(k_pol=0.2) if w["polarity"] else tg.Spring2R(k_rep=2.0, r_rep=0.7, k_adh=0.5, r_adh=0.8)
    return tg.Simulation(tg.Settings(agent_count=n, capacity=cap, cutoff_distance=1.0, seed=1, pair_finder_settings=pf),
                         dims=w.get("dims", 3), pair_finder=w["finder"], integrator=w["integrator"],
                         com_fixer="global" if w["com"] else None, force=force, polarity=w["polarity"],
                         division=tg.Division(probability=w["division"], offset=0.25), device=device)


def make_oracle(w, n, mn, mx, steps=0, timing=False):
    import oracle

    cap = capacity_for(w, n, steps)
    finder = oracle.BINNED_GABRIEL if w["finder"] == "binned_gabriel" else oracle.BINNED_ALL_PAIRS
    return oracle.Oracle(finder=finder, integrator=oracle.HEUN if w["integrator"] == "heun" else oracle.EULER,
                         com_fix=w["com"], min_bounds=mn, max_bounds=mx, capacity=cap,
                         force=oracle.FORCE_POLARITY if w["polarity"] else oracle.FORCE_SPRING2R,
                         k_pol=0.2 if w["polarity"] else 0.0, has_polarity=w["polarity"],
                         division_probability=w["division"], division_offset=0.25, seed=1, timing=timing)


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None
        self._summary = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            # wait for the sampler's first line so that the timed region is covered
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 10.0 and self._lines() == 0 and self.proc.poll() is None:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        self.lo, self.hi = 0, None
        return self

    def _lines(self):
        try:
            with open(self.path) as f:
                return sum(1 for line in f if line.endswith("\n"))
        except OSError:
            return 0

    def start(self):
        """Mark the start of the timed region (samples before it are ignored)."""
        self.lo = self._lines()

    def stop(self):
        """Mark the end of the timed region, letting the sampler record at least one line inside it."""
        t0 = time.perf_counter()
        while self.proc and self._lines() <= self.lo and time.perf_counter() - t0 < 1.0:
            time.sleep(0.01)
        self.hi = self._lines()

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except Exception:
                self.proc.kill()

    def summary(self):
        """Median SM clock, maximum and throttle reasons inside the timed region (read once, then kept)."""
        if self._summary is None:
            self._summary = self._read()
        return self._summary

    def _read(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = [line for line in open(self.path) if line.endswith("\n")]
        for line in lines[self.lo:self.hi]:
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


def aggregate_over_ranks(total_s: float, cell_steps: float, device):
    """Job totals over the replicas: the slowest rank's time and the summed
    cell-steps (one process per GPU, no data-path collective)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return total_s, float(cell_steps)
    t = torch.tensor([total_s], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(cell_steps)], device=device, dtype=torch.float64)
    dist.all_reduce(c)
    return float(t.item()), float(c.item())


def pass_profile(workload: str, key: str):
    """A per-cell figure of one force-pass launch (DRAM bytes, warp instructions) from the committed ncu
    capture of this workload."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    try:
        return json.loads(p.read_text()).get(workload, {}).get(key)
    except Exception:
        return None


def traffic_per_pass(workload: str):
    return pass_profile(workload, "pass_dram_bytes_per_cell")


def cpu_steps(w, n, mn, mx, x, p, steps, threads, budget_s):
    """Time up to `steps` oracle steps (about budget_s seconds) after one warm-up step."""
    o = make_oracle(w, n, mn, mx, steps + 2, timing=True)
    o.set_state(x, p)
    t0 = time.perf_counter()
    o.step(w["dt"], 1, threads)
    first = time.perf_counter() - t0
    k = max(1, min(steps, int(budget_s / max(first, 1e-4))))
    cs = 0
    t0 = time.perf_counter()
    for _ in range(k):
        cs += o.count
        o.step(w["dt"], 1, threads)
    dt = time.perf_counter() - t0
    return cs / dt, k, dt


def run_reference(args):
    """The reference's algorithm on the host cores: the oracle's C restatement with OpenMP."""
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    w = WORKLOADS[args.workload]
    if not w.get("cpu", True):
        print(json.dumps({"impl": "reference", "unavailable": "the reference's naive Delaunay finder does O(N^3) "
                                                              "work per cell; no bounded sample at this size"}))
        return 0
    n = args.cells or w["cells"]
    threads = os.cpu_count() or 1
    x, p, mn, mx = w["make"](n)
    v, k, dt = cpu_steps(w, n, mn, mx, x, p, max(args.steps, 1), threads, 60.0)
    line = {
        "impl": "reference", "metric": w["metric"], "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
        "warmup": 1, "ms_per_step": 1e3 * dt / max(k, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["desc"].format(n=n), "cells": n, "l2": "n/a (host)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{k} steps of the {n}-cell workload after 1 warm-up step ({dt:.1f} s, OpenMP)"},
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
    w = WORKLOADS[args.workload]
    n = args.cells or w["cells"]
    pol = w["polarity"]
    x, p, mn, mx = w["make"](n)
    # steps before the end-to-end leg re-uploads the initial state: warm-up,
    # timed, and the profiled run
    chunk = max(1, args.chunk)
    sim = make_sim(w, n, mn, mx, device=local,
                   steps=(args.warmup + args.steps) * chunk + 1 + min(args.steps * chunk, 100))
    stream = torch.cuda.ExternalStream(sim.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    xd = torch.from_numpy(x).to("cuda")
    pd = torch.from_numpy(p).to("cuda") if pol else None
    torch.cuda.synchronize()
    sim.set_state_device(xd.data_ptr(), pd.data_ptr() if pol else None, n)
    dt = w["dt"]

    for _ in range(args.warmup):
        sim.take_step(dt)
    sim.synchronize()

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    def timed_steps(k, per, profile):
        """k timed iterations of `per` simulation steps each, the L2 flushed
        before each; per-step milliseconds and cell-steps (the agent count
        before and after an iteration averaged over its steps)."""
        ms, cs = [], 0.0
        nb = sim.get_agent_count()
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            sim.take_step(dt, per)
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1) / per)
            if profile:
                for name, v in sim.last_step_profile():
                    kern.setdefault(name, []).append(v)
            na = sim.get_agent_count()
            cs += 0.5 * (nb + na) * per
            nb = na
        return ms, cs

    kern = {}
    with Clocks(local) as clocks:
        clocks.start()
        step_ms, cell_steps = timed_steps(args.steps, chunk, False)
        clocks.stop()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    # per-kernel CUDA events (event nodes inside the step graph) on a second,
    # shorter run of single steps: the kernel table and the shares
    sim.set_profiling(True)
    sim.take_step(dt)
    prof_ms, prof_cells = timed_steps(min(args.steps * chunk, 100), 1, True)
    sim.set_profiling(False)
    torch.cuda.synchronize()
    total_s, cell_steps_all = aggregate_over_ranks(sum(step_ms) * chunk / 1e3, cell_steps, "cuda")
    torch.cuda.synchronize()
    value = cell_steps_all / total_s
    kpl = sim.kernels_per_step()

    # End to end through the C ABI with host buffers: every step uploads the
    # state from pinned host memory, steps, and downloads the new state.
    e2e = None
    if not args.no_e2e:
        L = tg.load()
        cap = sim.desc.capacity
        D = w.get("dims", 3)
        hx = torch.empty((cap, D), dtype=torch.float32, pin_memory=True)
        hx.numpy()[:n] = x
        hp = torch.empty((cap, 2), dtype=torch.float32, pin_memory=True) if pol else None
        if pol:
            hp.numpy()[:n] = p
        nn = ctypes.c_uint(n)
        # the user-facing path: no per-kernel events; one untimed round trip
        # captures the step graph
        sim.set_profiling(False)
        tg._check(L.tecs_sim_upload(sim._h, ctypes.c_void_p(hx.data_ptr()),
                                    ctypes.c_void_p(hp.data_ptr()) if pol else None, n))
        tg._check(L.tecs_sim_step(sim._h, dt, 1))
        tg._check(L.tecs_sim_download(sim._h, ctypes.c_void_p(hx.data_ptr()),
                                      ctypes.c_void_p(hp.data_ptr()) if pol else None, ctypes.byref(nn)))
        hx.numpy()[:n] = x
        if pol:
            hp.numpy()[:n] = p
        nn = ctypes.c_uint(n)
        h2d = d2h = 0
        cs = 0
        t_up = t_rest = 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            m = nn.value
            ta = time.perf_counter()
            tg._check(L.tecs_sim_upload(sim._h, ctypes.c_void_p(hx.data_ptr()),
                                        ctypes.c_void_p(hp.data_ptr()) if pol else None, m))
            tb = time.perf_counter()
            h2d += m * (4 * D + (8 if pol else 0))
            tg._check(L.tecs_sim_step(sim._h, dt, 1))
            tg._check(L.tecs_sim_download(sim._h, ctypes.c_void_p(hx.data_ptr()),
                                          ctypes.c_void_p(hp.data_ptr()) if pol else None, ctypes.byref(nn)))
            t_up += tb - ta
            t_rest += time.perf_counter() - tb
            d2h += nn.value * (4 * D + (8 if pol else 0))
            cs += m
        t1 = time.perf_counter()
        e2e = {"value": cs / (t1 - t0), "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
               "d2h_bytes_per_step": int(d2h / args.steps),
               "ms_upload": 1e3 * t_up / args.steps, "ms_step_and_download": 1e3 * t_rest / args.steps,
               "note": "each step: pinned host state -> device (tecs_sim_upload, synchronous), tecs_sim_step, "
                       "device -> pinned host state (tecs_sim_download, synchronous)"}

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    hbm, peak_kind = peaks()
    n_avg = cell_steps / max(args.steps * chunk, 1)
    n_prof = prof_cells / max(len(prof_ms), 1)
    pass_bytes, pass_s_prof, pass_launches = 0.0, 0.0, 0
    for name, v in kern.items():
        if name in PASS_BYTES:
            b = PASS_BYTES[name][0] + (PASS_BYTES[name][1] if pol else 0)
            pass_bytes += b * n_prof * len(v)
            pass_s_prof += sum(v) / 1e3
            pass_launches += len(v)
    # The pass's launch time in the TIMED run: its share of the profiled
    # step (per-kernel events) times the timed step; the event nodes of the
    # profiled run add their own overhead, stated beside it.
    prof_kernel_s = sum(sum(v) for v in kern.values()) / 1e3
    share = pass_s_prof / prof_kernel_s if prof_kernel_s else float("nan")
    steps_prof = max(len(prof_ms), 1)
    launches_per_step = pass_launches / steps_prof
    timed_step_s = statistics.mean(step_ms) / 1e3
    pass_launch_s = share * timed_step_s / max(launches_per_step, 1e-9)
    bytes_per_launch = pass_bytes / max(pass_launches, 1)
    achieved = bytes_per_launch * (n_avg / n_prof) / pass_launch_s / 1e9 if pass_launch_s else float("nan")
    tpc = traffic_per_pass(args.workload)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": (tpc * n_avg if tpc else None),
                "kernel": ("one-launch Euler step (k_step_small: bin sort + pair finding + force + integrator)"
                           if "k_step_small" in kern else
                           "force pass (k_pass_*: pair finding + force + fused integrator epilogue)"),
                "bytes_per_launch": bytes_per_launch * n_avg / n_prof,
                "peak_kind": f"{peak_kind} hbm_gbs", "avg_launch_ms": 1e3 * pass_launch_s,
                "avg_launch_ms_basis": "the pass's share of the profiled step (per-kernel CUDA events) times "
                                       "the timed step",
                "profiled_launch_ms": 1e3 * pass_s_prof / max(pass_launches, 1),
                "profiled_step_over_timed_step": (prof_kernel_s / steps_prof) / timed_step_s}
    pass_s = pass_launch_s * launches_per_step * len(step_ms) * chunk
    pass_launches_timed = launches_per_step * len(step_ms) * chunk
    # The pass is bound by instruction issue, not HBM: warp instructions per launch (ncu count per cell x
    # cells) over the live launch time, against SMs x 4 schedulers x the sampled SM clock.
    ipc = pass_profile(args.workload, "pass_warp_inst_per_cell")
    issue_roofline = None
    if ipc and pass_s:
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = (clocks.summary() or {}).get("sm_mhz") or 2070.0
        ipeak = sms * 4 * mhz * 1e6
        iach = ipc * n_avg * pass_launches_timed / pass_s
        issue_roofline = {"bound": "issue", "achieved": iach, "peak": ipeak, "unit": "warp instructions/s",
                          "frac": iach / ipeak, "inst_per_cell": ipc,
                          "peak_basis": f"{sms} SMs x 4 schedulers x {mhz:.0f} MHz (sampled)",
                          "source": "profiles/traffic.json (ncu smsp__inst_executed.sum of one launch)"}
    step_achieved = w["step_bytes"] * n_avg / (statistics.mean(step_ms) / 1e3) / 1e9
    kernel_table = {k: {"launches": len(v), "mean_ms": statistics.mean(v), "share": sum(v) / max(sum(prof_ms), 1e-9)}
                    for k, v in kern.items()}
    cpu = None
    if not args.no_cpu_baseline and world == 1 and w.get("cpu", True):
        threads = os.cpu_count() or 1
        v, k, sec = cpu_steps(w, n, mn, mx, x, p, 1000, threads, 15.0)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{k} steps of the {n}-cell workload after 1 warm-up step ({sec:.1f} s, OpenMP)"}
    ensemble = None
    if world == 1 and args.workload == "spheroid" and not args.no_ensemble:
        ensemble = ensemble_comparison(args, local)
    line = {
        "metric": w["metric"], "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms),
        "ms_per_timed_step": statistics.mean(step_ms) * chunk, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": w["desc"].format(n=n), "cells": n, "capacity": sim.desc.capacity,
                   "sim_steps_per_timed_step": chunk, "sim_steps_timed": args.steps * chunk,
                   "l2": f"flushed (256 MiB memset) before each timed step of {chunk} simulation steps",
                   "parallelism": f"replicas x{world}"},
        "roofline": roofline,
        "step_roofline": {"bytes_per_cell": w["step_bytes"], "achieved": step_achieved,
                          "frac": step_achieved / hbm},
        "issue_roofline": issue_roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": kpl * args.steps * chunk,
        "kernels": kernel_table,
        "clocks": clocks.summary(),
        "ensemble": ensemble,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def ensemble_comparison(args, device, steps: int = 300):
    """The 256-simulation ensemble (cells log-uniform in [500, 200000], seed 2;
    half Gabriel, half binned all-pairs; Heun dt 0.05) for its 300 steps:
    the batched engine against the plain drop-in run one simulation after
    another, both timed with the state resident on the device."""
    from tecs_gb300 import batched

    members = batched.ensemble(256, 2)
    cells = sum(len(m.x) for m in members)
    scales, _ = batched.autotune(members)
    eng, _ = batched.build_engine(members, scales, device=device)
    t_b = batched.time_engine_steps(eng, steps, warmup=3)
    kpl = eng.kernels_per_step()
    eng.close()
    t_p = batched.run_plain_steps_only(members, steps)
    v_b, v_p = cells * steps / t_b, cells * steps / t_p
    return {"metric": "cell-steps/s, 256-simulation ensemble", "unit": UNIT, "steps": steps, "cells": cells,
            "batched": {"value": v_b, "ms_per_step": 1e3 * t_b / steps, "gpu_launches": kpl * steps},
            "plain_sequential": {"value": v_p, "ms_per_step_all_sims": 1e3 * t_p / steps},
            "speedup_batched_vs_plain": v_b / v_p, "bin_size_scale": scales}


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
    ap.add_argument("--steps", type=int, default=20,
                    help="timed steps, each of --chunk simulation steps (default 20 x 10: the spheroid "
                         "configuration's 200 steps)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cells", type=int, default=0, help="cell count (default: the workload's)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble comparison of the default run")
    ap.add_argument("--chunk", type=int, default=10,
                    help="simulation steps per timed step (the L2 is flushed between timed steps)")
    ap.add_argument("--workload", default="spheroid",
                    choices=["spheroid", "sheet", "small", "delaunay", "delaunay3d", "ensemble", "served"])
    ap.add_argument("--sims", type=int, default=256)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--requests", type=int, default=200, help="served workload: number of requests")
    ap.add_argument("--time-scale", type=float, default=1.0, help="served workload: arrival-time compression")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        if args.workload not in WORKLOADS:
            print(json.dumps({"impl": "reference", "unavailable": f"the reference has no {args.workload} form"}))
            return 0
        return run_reference(args)
    if args.workload == "ensemble":
        return run_ensemble(args)
    if args.workload == "served":
        from tecs_gb300 import served
        return served.bench_main(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
