"""Batched ensemble: many independent simulations in one engine step.

The ensemble workload is 256 simulations with cell counts log-uniform in
[500, 200000] (seed 2), each a ball at density 1, per-simulation spring
constants k_rep ~ U[1.5, 2.5], k_adh ~ U[0.3, 0.7], half of them with the
Gabriel finder and half with plain binned all-pairs, Heun dt = 0.05.  The
batched form runs them all in one Engine; the plain form runs the drop-in
Simulation on each one after the other.  An autotuner picks the bin size per
size class by timing short runs of copies.
"""
from __future__ import annotations

import json
import math
import os
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Dict, List, Optional

import numpy as np

import tecs_gb300 as tg
from tecs_gb300 import workloads as wl
from tecs_gb300.engine import Engine, bins_needed

CACHE = Path(os.environ.get("TECS_TUNE_CACHE", Path(__file__).resolve().parent / "_build" / "autotune.json"))


@dataclass
class Member:
    x: np.ndarray
    settings: tg.Settings
    finder: str
    integrator: str
    force: tg.Spring2R
    spec: wl.SimSpec

    def desc(self, bin_size_scale: float = 1.0) -> tg.SimDesc:
        d = tg.make_desc(self.settings, pair_finder=self.finder, integrator=self.integrator, force=self.force)
        d.bin_size_scale = bin_size_scale
        return d


def ensemble(n_sims: int = 256, seed: int = 2, lo: int = 500, hi: int = 200_000) -> List[Member]:
    out = []
    for sp in wl.ensemble(n_sims, seed, lo, hi):
        x = wl.ball(sp.n, sp.seed)
        mn, mx = wl.bounds_for(x)
        settings = tg.Settings(agent_count=sp.n, capacity=sp.n,
                               pair_finder_settings=tg.PairFinderSettings(min_bounds=mn, max_bounds=mx))
        out.append(Member(x, settings, "binned_gabriel" if sp.gabriel else "binned_all_pairs", "heun",
                          tg.Spring2R(k_rep=sp.k_rep, k_adh=sp.k_adh), sp))
    return out


def size_class(n: int) -> str:
    return "small" if n < 5_000 else ("medium" if n < 50_000 else "large")


def build_engine(members: List[Member], scales: Optional[Dict[str, float]] = None, device: int = 0):
    """One engine holding every member; scales: bin-size scale per size class, and optionally the
    passes' threads per block under "pass_threads" (autotune's result)."""
    scales = scales or {}
    descs = [m.desc(scales.get(size_class(len(m.x)), 1.0)) for m in members]
    cells = sum(len(m.x) for m in members)
    bins = sum(bins_needed(d) for d in descs)
    eng = Engine(cell_capacity=cells + 1024, bin_capacity=bins + 1024, max_sims=len(members) + 8, device=device)
    slots = [eng.add(d, m.x) for d, m in zip(descs, members)]
    if scales.get("pass_threads"):
        eng.set_pass_threads(int(scales["pass_threads"]))
    return eng, slots


def time_engine_steps(eng: Engine, steps: int, warmup: int = 2, dt: float = 0.05):
    import torch

    stream = torch.cuda.ExternalStream(eng.stream)
    eng.step(dt, warmup)
    eng.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    eng.step(dt, steps)
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3


def autotune(members: List[Member], candidates=(1.0, 1.25, 1.5), steps: int = 4, use_cache: bool = True,
             thread_candidates=(64, 96, 128)):
    """Bin-size scale per size class, then the force passes' threads per block, that minimise the
    batched step time.

    Each scale is timed on a fresh engine holding the members of that size class
    only; then the whole ensemble, at the chosen scales, is timed at each block
    size (chosen["pass_threads"]).  Results are cached per (class, cell count
    bucket, finder mix) and per ensemble.
    """
    key_of = lambda cls, ms: f"{cls}:{int(math.log2(max(1, sum(len(m.x) for m in ms))))}:" \
                             f"{sum(m.finder == 'binned_gabriel' for m in ms)}/{len(ms)}"
    cache = {}
    if use_cache and CACHE.exists():
        try:
            cache = json.loads(CACHE.read_text())
        except Exception:
            cache = {}
    chosen, timings = {}, {}
    for cls in ("small", "medium", "large"):
        ms = [m for m in members if size_class(len(m.x)) == cls]
        if not ms:
            continue
        key = key_of(cls, ms)
        if key in cache:
            chosen[cls] = cache[key]["scale"]
            timings[cls] = cache[key]["timings"]
            continue
        res = {}
        for sc in candidates:
            eng, _ = build_engine(ms, {cls: sc})
            res[str(sc)] = time_engine_steps(eng, steps, warmup=1)
            eng.close()
        best = min(res, key=res.get)
        chosen[cls] = float(best)
        timings[cls] = res
        cache[key] = {"scale": float(best), "timings": res}
    if thread_candidates:
        key = "threads:" + ",".join(f"{cls}={chosen[cls]}" for cls in sorted(chosen)) + ":" + key_of("all", members)
        if key in cache:
            chosen["pass_threads"] = cache[key]["threads"]
            timings["pass_threads"] = cache[key]["timings"]
        else:
            eng, _ = build_engine(members, chosen)
            res = {}
            for t in thread_candidates:
                eng.set_pass_threads(t)
                res[str(t)] = time_engine_steps(eng, steps, warmup=1)
            eng.close()
            best = min(res, key=res.get)
            chosen["pass_threads"] = int(best)
            timings["pass_threads"] = res
            cache[key] = {"threads": int(best), "timings": res}
    if use_cache:
        CACHE.parent.mkdir(parents=True, exist_ok=True)
        CACHE.write_text(json.dumps(cache, indent=1, sort_keys=True))
    return chosen, timings


def run_plain(members: List[Member], steps: int, dt: float = 0.05):
    """The plain drop-in on each simulation, one after the other; seconds."""
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for m in members:
        s = tg.Simulation(m.settings, pair_finder=m.finder, integrator=m.integrator, force=m.force)
        s.set_state(m.x)
        s.take_step(dt, steps)
        s.synchronize()
        s.close()
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def run_plain_steps_only(members: List[Member], steps: int, dt: float = 0.05, warmup: int = 1):
    """Plain drop-in, timing only the stepping (set-up and upload excluded); seconds."""
    import torch

    sims = []
    for m in members:
        s = tg.Simulation(m.settings, pair_finder=m.finder, integrator=m.integrator, force=m.force)
        s.set_state(m.x)
        s.take_step(dt, warmup)
        sims.append(s)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in sims:
        s.take_step(dt, steps)
        s.synchronize()
    t = time.perf_counter() - t0
    for s in sims:
        s.close()
    return t
