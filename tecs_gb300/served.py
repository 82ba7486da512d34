"""Served form: a continuous-batching request loop over the engine.

Requests (simulation shape, model, integrator, step count) arrive on a
Poisson clock.  The loop admits a waiting request as soon as the engine has
free cells and a free run of bins for it (the engine's capacity is sized from
the GPU's free HBM), so requests that arrive while others are on the GPU join
the very next step and share every step's kernel launches with them.  Each
simulation's state stays on the device; every `snapshot_every` steps it is
unpacked on the device and copied to pinned host memory on a side stream, and
a writer thread stores it (HDF5 via tecs_gb300.h5, with the XDMF sidecar when
the sink is given the step's time) without stalling the steps.
A simulation that reaches its step count is downloaded, retired, and its
time-to-completion (arrival -> result on the host) recorded.

An engine advances all its resident simulations in lockstep, so a small
request sharing an engine with a large one pays the large one's step time for
each of its steps.  With size classes the server keeps one engine (a lane) per
class -- e.g. requests up to 50k cells in one, the rest in another -- each on
its own stream and paced by its own step events, so small requests progress
at their own rate while the large ones run alongside on the same GPU.
"""
from __future__ import annotations

import collections
import ctypes
import json
import math
import os
import queue
import threading
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable, Dict, List, Optional

import numpy as np

import tecs_gb300 as tg
from tecs_gb300 import workloads as wl
from tecs_gb300.engine import Engine, bins_needed

IN_FLIGHT = 2  # steps a lane may have queued on the GPU
# the served bench's lanes: requests up to 50k cells in an engine with a tenth of the capacity
BENCH_SIZE_CLASSES = [(50_000, 0.1), (None, 0.9)]
BYTES_PER_CELL = 140  # device bytes the engine keeps per cell (positions, deltas, polarity, sort scratch)
BYTES_PER_BIN = 8


def request_sim(req: wl.Request, max_cells: Optional[int] = None):
    """(positions, polarity, desc) for a request: a density-1 ball, or a polarised sheet."""
    n = req.n if max_cells is None else min(req.n, max_cells)
    if req.model == "polarity":
        x = wl.sheet(n, req.seed)
        p = wl.outward_polarity(x, req.seed)
        force = tg.PolaritySpring(k_pol=0.2)
    else:
        x = wl.ball(n, req.seed)
        p = None
        force = tg.Spring2R()
    mn, mx = wl.bounds_for(x)
    settings = tg.Settings(agent_count=n, capacity=n,
                           pair_finder_settings=tg.PairFinderSettings(min_bounds=mn, max_bounds=mx))
    d = tg.make_desc(settings, pair_finder="binned_gabriel", integrator=req.integrator, force=force,
                     polarity=p is not None)
    return x, p, d, settings, force


@dataclass
class Live:
    req: wl.Request
    slot: int
    n: int
    has_pol: bool
    steps_done: int = 0
    admitted_at: float = 0.0
    req_index: int = -1


@dataclass
class Lane:
    """One engine of the server and the requests it serves."""
    engine: Engine
    max_req_cells: Optional[int]  # requests up to this many cells (None: any)
    cell_capacity: int
    bin_capacity: int
    live: Dict[int, Live] = field(default_factory=dict)
    waiting: collections.deque = field(default_factory=collections.deque)
    stage_next: int = 0
    pending: collections.deque = field(default_factory=collections.deque)  # events of queued steps

    def takes(self, n: int) -> bool:
        return self.max_req_cells is None or n <= self.max_req_cells


@dataclass
class Result:
    index: int
    n: int
    steps: int
    arrival: float
    admitted: float
    completed: float
    positions: Optional[np.ndarray] = None
    polarity: Optional[np.ndarray] = None

    @property
    def latency(self):
        return self.completed - self.arrival


class SnapshotWriter(threading.Thread):
    """Waits for each snapshot's copy event, then hands the pinned buffer to the sink."""

    def __init__(self, sink: Optional[Callable] = None, ready: Callable = Engine.event_ready,
                 destroy: Callable = Engine.event_destroy):
        super().__init__(daemon=True)
        self.q = queue.Queue()
        self.sink = sink
        self.ready, self.destroy = ready, destroy
        self.written = 0
        self.errors: List[str] = []

    def run(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            ev, req_index, step, pos, pol, release = item
            while not self.ready(ev):
                time.sleep(0.0002)
            self.destroy(ev)
            try:
                if self.sink:
                    self.sink(req_index, step, pos, pol)
                self.written += 1
            except Exception as exc:  # a failing sink fails that snapshot, not the server
                self.errors.append(f"request {req_index} step {step}: {exc}")
            release()


class PinnedPool:
    """Reusable pinned host buffers (so snapshots do not allocate per copy)."""

    def __init__(self):
        import torch

        self.torch = torch
        self.free: Dict[tuple, list] = collections.defaultdict(list)
        self.lock = threading.Lock()

    def get(self, n: int, width: int):
        key = (n, width)
        with self.lock:
            if self.free[key]:
                return self.free[key].pop()
        return self.torch.empty((n, width), dtype=self.torch.float32, pin_memory=True)

    def put(self, t):
        with self.lock:
            self.free[(t.shape[0], t.shape[1])].append(t)


class Server:
    """size_classes: [(largest request in cells, or None for any; share of the capacity)], one engine
    (lane) per class, in order; None keeps a single engine for every request."""

    def __init__(self, cell_capacity: int, bin_capacity: int, max_sims: int = 1024, snapshot_every: int = 100,
                 dt: float = 0.05, sink: Optional[Callable] = None, keep_results: bool = False, device: int = 0,
                 size_classes=None, steps_per_issue: int = 1):
        self.device = device
        classes = size_classes or [(None, 1.0)]
        if classes[-1][0] is not None:
            raise ValueError("the last size class must take any request (None)")
        self.lanes: List[Lane] = []
        for max_cells, share in classes:
            c, b = max(int(cell_capacity * share), 1), max(int(bin_capacity * share), 1)
            self.lanes.append(Lane(self._engine(c, b, max_sims), max_cells, c, b))
        self.engine = self.lanes[0].engine
        self.streams = [self._stream(l) for l in self.lanes]
        self.cell_capacity = cell_capacity
        self.bin_capacity = bin_capacity
        self.dt = dt
        self.snapshot_every = snapshot_every
        self.writer = SnapshotWriter(sink, *self._event_ops())
        self.writer.start()
        self.pool = self._pool()
        self.keep_results = keep_results
        self.cell_steps = 0
        self.steps = 0
        # up to this many steps per engine call, never past a resident request's next snapshot or end
        self.steps_per_issue = max(1, int(steps_per_issue))

    def lane_for(self, n: int) -> Lane:
        return next(l for l in self.lanes if l.takes(n))

    # the device-facing pieces: a lane's engine and stream, an event recorded after its queued steps, the
    # readiness test of a snapshot copy's event, pinned buffers
    def _engine(self, cells: int, bins: int, max_sims: int):
        return Engine(cells, bins, max_sims, self.device)

    def _stream(self, lane: Lane):
        import torch

        return torch.cuda.ExternalStream(lane.engine.stream, device=torch.device("cuda", self.device))

    def _record(self, stream):
        import torch

        ev = torch.cuda.Event()
        ev.record(stream)
        return ev

    def _event_ops(self):
        return Engine.event_ready, Engine.event_destroy

    def _pool(self):
        return PinnedPool()

    @staticmethod
    def capacity_from_free_hbm(fraction: float = 0.5, bins_per_cell: float = 3.0):
        import torch

        free, _ = torch.cuda.mem_get_info()
        budget = free * fraction
        cells = int(budget / (BYTES_PER_CELL + bins_per_cell * BYTES_PER_BIN))
        return max(cells, 1 << 16), int(max(cells, 1 << 16) * bins_per_cell)

    def _snapshot(self, lane: Lane, live: Live, step: int):
        pos = self.pool.get(live.n, 3)
        pol = self.pool.get(live.n, 2) if live.has_pol else None
        if lane.stage_next + live.n > lane.cell_capacity:
            lane.stage_next = 0
            lane.engine.synchronize()  # staging reused: let queued copies finish
        ev = lane.engine.snapshot_async(live.slot, pos.data_ptr(), None if pol is None else pol.data_ptr(),
                                        lane.stage_next)
        lane.stage_next += live.n

        def release(pos=pos, pol=pol):
            self.pool.put(pos)
            if pol is not None:
                self.pool.put(pol)

        self.writer.q.put((ev, live.req_index, step, pos.numpy(), None if pol is None else pol.numpy(), release))

    def run(self, requests: List[wl.Request], time_scale: float = 1.0, max_cells: Optional[int] = None,
            prebuild: bool = True, resume: Optional[Dict[int, tuple]] = None):
        """Serve the requests; arrival times are divided by time_scale.  Returns the results.

        resume: {request index: (step, positions, polarity or None)} -- such a request starts from that
        state (a snapshot, h5.last_snapshot) and runs only its remaining steps; its snapshots and its end
        fall on the same steps as in an uninterrupted run, and so does its result (the state is the
        positions and polarities, in cell-id order)."""
        resume = resume or {}
        reqs = sorted(enumerate(requests), key=lambda kv: kv[1].arrival_s)
        built = {}
        for idx, r in reqs:
            sim = request_sim(r, max_cells)
            if idx in resume:
                step, pos, pol = resume[idx]
                if len(pos) != len(sim[0]) or (pol is None) != (sim[1] is None) or not 0 <= step <= r.steps:
                    raise ValueError(f"resume state of request {idx} does not match the request")
                sim = (np.ascontiguousarray(pos, np.float32),
                       None if pol is None else np.ascontiguousarray(pol, np.float32)) + tuple(sim[2:])
            lane = self.lane_for(len(sim[0]))
            if len(sim[0]) > lane.cell_capacity or bins_needed(sim[2]) > lane.bin_capacity:
                raise ValueError(f"request {idx} ({len(sim[0])} cells, {bins_needed(sim[2])} bins) "
                                 f"exceeds its engine ({lane.cell_capacity} cells, {lane.bin_capacity} bins)")
            if prebuild:
                built[idx] = sim
        results: List[Result] = []
        arrival = {idx: r.arrival_s / time_scale for idx, r in reqs}
        k = 0
        t0 = time.perf_counter()
        while k < len(reqs) or any(l.waiting or l.live for l in self.lanes):
            now = time.perf_counter() - t0
            while k < len(reqs) and arrival[reqs[k][0]] <= now:
                idx = reqs[k][0]
                n = len(built[idx][0]) if idx in built else len(request_sim(requests[idx], max_cells)[0])
                self.lane_for(n).waiting.append(idx)
                k += 1
            # admission, per lane: first come, first served, while cells and bins are free
            for lane in self.lanes:
                while lane.waiting:
                    idx = lane.waiting[0]
                    x, p, d, _, _ = built[idx] if idx in built else request_sim(requests[idx], max_cells)
                    free_cells, free_bins = lane.engine.free()
                    if len(x) > free_cells or bins_needed(d) > free_bins:
                        break
                    lane.waiting.popleft()
                    slot = lane.engine.add(d, x, p)
                    lane.live[slot] = Live(requests[idx], slot, len(x), p is not None,
                                           resume[idx][0] if idx in resume else 0, time.perf_counter() - t0, idx)
                if lane.waiting and not lane.live:  # an idle engine holds nothing: the head must fit
                    raise RuntimeError(f"request {lane.waiting[0]} cannot be admitted into an idle engine")
            # resumed requests that were already complete
            for lane in self.lanes:
                for slot in [s_ for s_, lv in lane.live.items() if lv.steps_done >= lv.req.steps]:
                    lv = lane.live.pop(slot)
                    xf, pf = lane.engine.download(slot)
                    lane.engine.remove(slot)
                    res = Result(lv.req_index, lv.n, lv.req.steps, arrival[lv.req_index], lv.admitted_at,
                                 time.perf_counter() - t0)
                    if self.keep_results:
                        res.positions, res.polarity = xf, pf
                    results.append(res)
            if not any(l.live for l in self.lanes):
                if k < len(reqs):
                    time.sleep(max(0.0, min(0.01, arrival[reqs[k][0]] - (time.perf_counter() - t0))))
                continue
            # one step of every resident simulation of each lane with fewer than IN_FLIGHT steps queued
            # (each lane keeps its GPU queue fed at its own pace)
            issued = False
            for lane, stream in zip(self.lanes, self.streams):
                while lane.pending and lane.pending[0].query():
                    lane.pending.popleft()
                if not lane.live or len(lane.pending) >= IN_FLIGHT:
                    continue
                kk = self.steps_per_issue
                for lv in lane.live.values():
                    to_snap = self.snapshot_every - lv.steps_done % self.snapshot_every
                    kk = min(kk, lv.req.steps - lv.steps_done, to_snap)
                kk = max(kk, 1)
                lane.engine.step(self.dt, kk)
                lane.pending.append(self._record(stream))
                issued = True
                self.steps += kk
                for lv in lane.live.values():
                    lv.steps_done += kk
                    self.cell_steps += lv.n * kk
                done = []
                for slot, lv in lane.live.items():
                    if lv.steps_done % self.snapshot_every == 0 and lv.steps_done < lv.req.steps:
                        self._snapshot(lane, lv, lv.steps_done)
                    if lv.steps_done >= lv.req.steps:
                        done.append(slot)
                for slot in done:
                    lv = lane.live.pop(slot)
                    xf, pf = lane.engine.download(slot)
                    lane.engine.remove(slot)
                    res = Result(lv.req_index, lv.n, lv.req.steps, arrival[lv.req_index], lv.admitted_at,
                                 time.perf_counter() - t0)
                    if self.keep_results:
                        res.positions, res.polarity = xf, pf
                    results.append(res)
            if not issued:
                time.sleep(0.00005)
        for lane in self.lanes:
            lane.engine.synchronize()
        self.makespan = time.perf_counter() - t0
        return results

    def close(self):
        self.writer.q.put(None)
        self.writer.join(timeout=60)
        for lane in self.lanes:
            lane.engine.close()


class _ServeDesc(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("cell_capacity", ctypes.c_uint), ("bin_capacity", ctypes.c_uint),
                ("max_sims", ctypes.c_uint), ("dt", ctypes.c_double), ("snapshot_every", ctypes.c_uint),
                ("snapshot_dir", ctypes.c_char_p), ("n_lanes", ctypes.c_uint),
                ("lane_max_cells", ctypes.c_uint * 4), ("lane_share", ctypes.c_float * 4),
                ("steps_per_issue", ctypes.c_uint), ("in_flight", ctypes.c_uint)]


class _ServeResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("tag", ctypes.c_uint64), ("cells", ctypes.c_uint), ("steps", ctypes.c_uint),
                ("arrival_s", ctypes.c_double), ("admitted_s", ctypes.c_double), ("completed_s", ctypes.c_double)]


class _ServeStats(ctypes.Structure):
    _fields_ = [("cell_steps", ctypes.c_ulonglong), ("engine_steps", ctypes.c_ulonglong),
                ("snapshots_written", ctypes.c_ulonglong), ("snapshot_errors", ctypes.c_ulonglong),
                ("submitted", ctypes.c_uint), ("completed", ctypes.c_uint), ("resident", ctypes.c_uint),
                ("waiting", ctypes.c_uint)]


def _serve_lib():
    L = tg.load()
    if getattr(L, "_serve_bound", False):
        return L
    vp = ctypes.c_void_p
    L.tecs_serve_desc_default.argtypes = [ctypes.POINTER(_ServeDesc)]
    L.tecs_serve_create.argtypes = [ctypes.POINTER(_ServeDesc), ctypes.POINTER(vp)]
    L.tecs_serve_submit.argtypes = [vp, ctypes.POINTER(tg.SimDesc), vp, vp, ctypes.c_uint, ctypes.c_uint,
                                    ctypes.c_uint, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    L.tecs_serve_poll.argtypes = [vp, ctypes.POINTER(_ServeResult), ctypes.c_uint, ctypes.POINTER(ctypes.c_uint)]
    L.tecs_serve_fetch.argtypes = [vp, ctypes.c_uint64, vp, vp, ctypes.POINTER(ctypes.c_uint)]
    L.tecs_serve_drain.argtypes = [vp, ctypes.c_double]
    L.tecs_serve_stats_get.argtypes = [vp, ctypes.POINTER(_ServeStats)]
    L.tecs_serve_destroy.argtypes = [vp]
    for name in ("tecs_serve_desc_default", "tecs_serve_create", "tecs_serve_submit", "tecs_serve_poll",
                 "tecs_serve_fetch", "tecs_serve_drain", "tecs_serve_stats_get", "tecs_serve_destroy"):
        getattr(L, name).restype = ctypes.c_int
    L._serve_bound = True
    return L


class NativeServer:
    """The served loop of the library (include/tecs_gpu.h, tecs_serve_*): the same admission, lanes,
    multi-step issue, snapshots and retirement as Server, run by a server thread in the library, with
    snapshots written as HDF5 by its own writer thread (<snapshot_dir>/request_<index>.h5, the request's
    index in the list, as SnapshotSink names them; a resumed request starts a new file).  This thread only
    submits requests at their arrival times and collects the results."""

    def __init__(self, cell_capacity: int, bin_capacity: int, max_sims: int = 1024, snapshot_every: int = 100,
                 dt: float = 0.05, snapshot_dir=None, keep_results: bool = False, device: int = 0,
                 size_classes=None, steps_per_issue: int = 1, in_flight: int = IN_FLIGHT):
        L = _serve_lib()
        classes = size_classes or [(None, 1.0)]
        if classes[-1][0] is not None:
            raise ValueError("the last size class must take any request (None)")
        d = _ServeDesc()
        tg._check(L.tecs_serve_desc_default(ctypes.byref(d)))
        d.device = device
        d.cell_capacity = int(cell_capacity)
        d.bin_capacity = int(bin_capacity)
        d.max_sims = int(max_sims)
        d.dt = float(dt)
        d.snapshot_every = int(snapshot_every)
        self._dir = None if snapshot_dir is None else str(snapshot_dir).encode()
        d.snapshot_dir = self._dir
        d.n_lanes = len(classes)
        for k, (m, share) in enumerate(classes):
            d.lane_max_cells[k] = 0 if m is None else int(m)
            d.lane_share[k] = float(share)
        d.steps_per_issue = int(steps_per_issue)
        d.in_flight = int(in_flight)
        h = ctypes.c_void_p()
        tg._check(L.tecs_serve_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.size_classes = classes
        self.dt = dt
        self.keep_results = keep_results
        self.cell_steps = 0
        self.steps = 0
        self.makespan = 0.0
        self.written = 0

    def run(self, requests: List[wl.Request], time_scale: float = 1.0, max_cells: Optional[int] = None,
            resume: Optional[Dict[int, tuple]] = None, timeout_s: float = 3600.0):
        """Serve the requests (arrival times divided by time_scale); returns the results, as Server.run."""
        L = _serve_lib()
        resume = resume or {}
        reqs = sorted(enumerate(requests), key=lambda kv: kv[1].arrival_s)
        built = {}
        for idx, r in reqs:
            x, p, d, _, _ = request_sim(r, max_cells)
            start = 0
            if idx in resume:
                start, pos, pol = resume[idx]
                if len(pos) != len(x) or (pol is None) != (p is None) or not 0 <= start <= r.steps:
                    raise ValueError(f"resume state of request {idx} does not match the request")
                x = np.ascontiguousarray(pos, np.float32)
                p = None if pol is None else np.ascontiguousarray(pol, np.float32)
            built[idx] = (np.ascontiguousarray(x, np.float32),
                          None if p is None else np.ascontiguousarray(p, np.float32), d, start)
        ids = {}
        t0 = time.perf_counter()
        for idx, r in reqs:
            wait = r.arrival_s / time_scale - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            x, p, d, start = built[idx]
            rid = ctypes.c_uint64()
            tg._check(L.tecs_serve_submit(self._h, ctypes.byref(d), tg._ptr(x), tg._ptr(p), len(x), r.steps, start,
                                          idx, ctypes.byref(rid)))
            ids[rid.value] = idx
        tg._check(L.tecs_serve_drain(self._h, float(timeout_s)))
        self.makespan = time.perf_counter() - t0
        results: List[Result] = []
        buf = (_ServeResult * 256)()
        n = ctypes.c_uint()
        while True:
            tg._check(L.tecs_serve_poll(self._h, buf, 256, ctypes.byref(n)))
            if n.value == 0:
                break
            for k in range(n.value):
                rr = buf[k]
                idx = ids[rr.id]
                res = Result(idx, rr.cells, requests[idx].steps, rr.arrival_s, rr.admitted_s, rr.completed_s)
                if self.keep_results:
                    x = np.empty((rr.cells, 3), np.float32)
                    p = np.empty((rr.cells, 2), np.float32) if built[idx][1] is not None else None
                    cnt = ctypes.c_uint()
                    tg._check(L.tecs_serve_fetch(self._h, rr.id, tg._ptr(x), tg._ptr(p), ctypes.byref(cnt)))
                    res.positions, res.polarity = x, p
                results.append(res)
        st = _ServeStats()
        tg._check(L.tecs_serve_stats_get(self._h, ctypes.byref(st)))
        self.cell_steps = st.cell_steps
        self.steps = st.engine_steps
        self.written = st.snapshots_written
        self.request_of = ids
        return sorted(results, key=lambda r: r.index)

    def close(self):
        if getattr(self, "_h", None):
            _serve_lib().tecs_serve_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def resume_points(directory, indices) -> Dict[int, tuple]:
    """{request index: (step, positions, polarity)} from the newest snapshots in `directory`, for the
    requests that have one."""
    from tecs_gb300 import h5

    out = {}
    for idx in indices:
        snap = h5.last_snapshot(directory, idx)
        if snap is not None:
            out[idx] = snap
    return out


def summarize(results: List[Result], makespan: float, cell_steps: int):
    lat = np.array([r.latency for r in results])
    return {
        "requests": len(results),
        "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
        "mean_s": float(lat.mean()) if len(lat) else None,
        "cell_steps_per_s": cell_steps / makespan if makespan > 0 else None,
        "makespan_s": makespan,
    }


def plain_sample(requests: List[wl.Request], every: int = 10, dt: float = 0.05):
    """The plain drop-in (one tecs_gb300.Simulation per request, one request
    after another, state set up outside the timing) on every `every`-th
    request of the stream.  Returns cell-steps/s, the sample's (cells, steps,
    seconds) rows."""
    import torch

    rows = []
    for r in requests[::every]:
        x, p, d, settings, force = request_sim(r)
        s = tg.Simulation(settings, pair_finder="binned_gabriel", integrator=r.integrator, force=force,
                          polarity=p is not None)
        s.set_state(x, p)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.take_step(dt, r.steps)
        s.synchronize()
        rows.append((len(x), r.steps, time.perf_counter() - t0))
        s.close()
    cs = sum(n * k for n, k, _ in rows)
    return cs / sum(t for _, _, t in rows), rows


def plain_fcfs_latency(requests: List[wl.Request], rows, time_scale: float = 1.0):
    """Time to completion of the same arrivals served by the plain path one
    request at a time, first come first served.  A request's run time is
    steps * (a + b * cells) (+ c per request), least-squares fitted to the
    measured sample rows."""
    A = np.array([[k, k * n, 1.0] for n, k, _ in rows])
    y = np.array([t for _, _, t in rows])
    coef, *_ = np.linalg.lstsq(A, y, rcond=None)
    coef = np.maximum(coef, 0.0)
    free_at, lat = 0.0, []
    for r in sorted(requests, key=lambda r: r.arrival_s):
        n = r.n
        t = coef[0] * r.steps + coef[1] * r.steps * n + coef[2]
        start = max(free_at, r.arrival_s / time_scale)
        free_at = start + t
        lat.append(free_at - r.arrival_s / time_scale)
    lat = np.array(lat)
    return {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "makespan_s": float(free_at), "model_s_per_step": [float(c) for c in coef]}


def bench_main(args):
    """bench.py --workload served: the served stream on one GPU."""
    import torch

    rank, world, local = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(
        os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    n_req = args.requests
    reqs = wl.served_stream(n_req, seed=3)
    cells, bins = Server.capacity_from_free_hbm(0.4)
    out_dir = Path(os.environ.get("TECS_SNAPSHOT_DIR", "/tmp/tecs_snapshots"))
    out_dir.mkdir(parents=True, exist_ok=True)
    dt = 0.05
    # the library's own loop (tecs_serve_*): server and HDF5 writer threads in C++
    srv = NativeServer(cells, bins, max_sims=4096, snapshot_every=100, dt=dt, snapshot_dir=out_dir,
                       size_classes=BENCH_SIZE_CLASSES, steps_per_issue=8)
    res = srv.run(reqs, time_scale=args.time_scale)
    summ = summarize(res, srv.makespan, srv.cell_steps)
    small = [r for r in res if r.n <= BENCH_SIZE_CLASSES[0][0]]
    large = [r for r in res if r.n > BENCH_SIZE_CLASSES[0][0]]
    by_class = {name: {"requests": len(rs), "p50_s": float(np.percentile([r.latency for r in rs], 50)),
                       "p99_s": float(np.percentile([r.latency for r in rs], 99))}
                for name, rs in (("small", small), ("large", large)) if rs}
    written = srv.written
    srv.close()
    plain_v, rows = plain_sample(reqs)
    plain_lat = plain_fcfs_latency(reqs, rows, args.time_scale)
    # capacity: the same stream with arrivals compressed 100 times (compute-bound)
    cap_srv = NativeServer(cells, bins, max_sims=4096, snapshot_every=0, dt=dt, snapshot_dir=None,
                           size_classes=BENCH_SIZE_CLASSES, steps_per_issue=8)
    cap_res = cap_srv.run(reqs, time_scale=100.0)
    cap = summarize(cap_res, cap_srv.makespan, cap_srv.cell_steps)
    cap_srv.close()
    line = {
        "metric": "cell-steps/s, served stream (continuous batching)", "value": summ["cell_steps_per_s"],
        "unit": "cell-steps/s", "n_gpus": 1, "steps": srv.steps, "warmup": 0,
        "ms_per_step": 1e3 * srv.makespan / max(srv.steps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n_req} requests, Poisson 20/s (seed 3) with arrivals compressed x{args.time_scale}, "
                               "cells log-uniform [1e3, 1e6], steps U[100, 1000], spring|polarity x euler|heun, "
                               "snapshots every 100 steps", "engine_cells": cells, "engine_bins": bins,
                   "size_classes": [{"max_request_cells": m, "capacity_share": f} for m, f in BENCH_SIZE_CLASSES],
                   "steps_per_issue": 8, "loop": "tecs_serve_* (server and HDF5 writer threads in the library)"},
        "latency": {"p50_s": summ["p50_s"], "p99_s": summ["p99_s"], "mean_s": summ["mean_s"],
                    "by_size_class": by_class},
        "capacity": {"value": cap["cell_steps_per_s"], "makespan_s": cap["makespan_s"],
                     "note": "the same requests with arrivals compressed x100 (no snapshots): compute-bound"},
        "plain_sequential": {"value": plain_v, "requests": len(rows),
                             "fcfs_latency_model": plain_lat,
                             "note": "every 10th request run alone through the plain path, one after another; "
                                     "fcfs_latency_model = the same arrivals served one at a time by the plain "
                                     "path, run times fitted to the sample"},
        "capacity_vs_plain": cap["cell_steps_per_s"] / plain_v,
        "snapshots_written": written, "makespan_s": srv.makespan,
    }
    print(json.dumps(line), flush=True)
    return 0
