"""The served loop's host logic on the CPU, over a stand-in engine.

The stand-in keeps each resident simulation's state on the host and advances
it by a fixed float32 map per step, so a request's result after k steps, and
its state at every snapshot, are known exactly.  The tests check the server's
bookkeeping around the engine calls:
- every request runs exactly its step count;
- snapshots fall on every multiple of `snapshot_every` below the end;
- multi-step issue never crosses a snapshot or a request's end;
- size classes route each request to its own lane;
- admission waits, first come first served, for free cells and bins;
- no lane queues more than IN_FLIGHT steps;
- a resumed request runs only its remaining steps and ends where the
  uninterrupted run does, and an appending sink leaves its snapshot files as
  one run's.
The same loop over the CUDA engine is covered by the GPU tests.
"""
import ctypes
import sys
from pathlib import Path

import numpy as np
import pytest
import torch

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from tecs_gb300 import served  # noqa: E402
from tecs_gb300 import workloads as wl  # noqa: E402
from tecs_gb300.engine import bins_needed  # noqa: E402

DT = 0.05


def advance(x, p):
    """One step of the stand-in dynamics (float32 throughout)."""
    x = (x * np.float32(0.999) + np.float32(DT) * np.float32(0.5)).astype(np.float32)
    if p is not None:
        p = (p + np.float32(DT) * np.float32(0.25)).astype(np.float32)
    return x, p


def advanced(x, p, k):
    for _ in range(k):
        x, p = advance(x, p)
    return x, p


class FakeEvent:
    """Done after `lag` queries, like a GPU that runs a little behind the host."""

    def __init__(self, lag=2):
        self.left = lag

    def query(self):
        self.left -= 1
        return self.left < 0


class FakeEngine:
    def __init__(self, cells, bins, max_sims):
        self.cells, self.bins, self.max_sims = cells, bins, max_sims
        self.sims = {}  # slot -> [positions, polarity, bins, steps taken]
        self.next_slot = 0
        self.adds, self.steps, self.snaps, self.downloads = [], [], [], []
        self.peak_cells = 0

    def free(self):
        return (self.cells - sum(len(v[0]) for v in self.sims.values()),
                self.bins - sum(v[2] for v in self.sims.values()))

    def add(self, desc, x, p=None):
        fc, fb = self.free()
        nb = bins_needed(desc)
        assert len(x) <= fc and nb <= fb and len(self.sims) < self.max_sims
        slot, self.next_slot = self.next_slot, self.next_slot + 1
        self.sims[slot] = [np.array(x, np.float32), None if p is None else np.array(p, np.float32), nb, 0]
        self.adds.append(len(x))
        self.peak_cells = max(self.peak_cells, self.cells - self.free()[0])
        return slot

    def step(self, dt, k=1):
        assert dt == DT and k >= 1
        self.steps.append(k)
        for v in self.sims.values():
            v[0], v[1] = advanced(v[0], v[1], k)
            v[3] += k

    def download(self, slot):
        x, p, _, taken = self.sims[slot]
        self.downloads.append((slot, taken))
        return x.copy(), None if p is None else p.copy()

    def remove(self, slot):
        del self.sims[slot]

    def snapshot_async(self, slot, pos_ptr, pol_ptr, stage_offset=0):
        x, p, _, taken = self.sims[slot]
        ctypes.memmove(pos_ptr, x.ctypes.data, x.nbytes)
        if pol_ptr is not None:
            ctypes.memmove(pol_ptr, p.ctypes.data, p.nbytes)
        self.snaps.append((slot, taken))
        return FakeEvent()

    def synchronize(self):
        pass

    def close(self):
        pass


class FakePool:
    def get(self, n, width):
        return torch.empty((n, width), dtype=torch.float32)

    def put(self, t):
        pass


class HostServer(served.Server):
    """The server with the stand-in engine, host buffers and host events."""

    def _engine(self, cells, bins, max_sims):
        return FakeEngine(cells, bins, max_sims)

    def _stream(self, lane):
        return lane

    def _record(self, lane):
        assert len(lane.pending) < served.IN_FLIGHT
        return FakeEvent()

    def _event_ops(self):
        return (lambda ev: ev.query()), (lambda ev: None)

    def _pool(self):
        return FakePool()


class Sink:
    def __init__(self, fail_at=None):
        self.got = {}
        self.fail_at = fail_at

    def __call__(self, req, step, pos, pol):
        if (req, step) == self.fail_at:
            raise OSError("disk full")
        self.got[(req, step)] = (pos.copy(), None if pol is None else pol.copy())


def stream(sizes_steps, models=("spring", "polarity")):
    return [wl.Request(arrival_s=0.001 * i, n=n, steps=k, model=models[i % len(models)],
                       integrator="heun" if i % 3 else "euler", seed=i)
            for i, (n, k) in enumerate(sizes_steps)]


def serve(reqs, cells=20_000, bins=200_000, sink=None, resume=None, **kw):
    srv = HostServer(cells, bins, max_sims=64, snapshot_every=kw.pop("snapshot_every", 10), dt=DT, sink=sink,
                     keep_results=True, **kw)
    try:
        res = srv.run(reqs, time_scale=100.0, resume=resume)
    finally:
        srv.close()
    return srv, {r.index: r for r in res}


def initial(req):
    x, p, *_ = served.request_sim(req)
    return x, p


REQS = [(300, 25), (1200, 40), (150, 7), (800, 30), (2000, 10), (60, 1)]


def check_results(reqs, res):
    assert sorted(res) == list(range(len(reqs)))
    for i, r in enumerate(reqs):
        ex, ep = advanced(*initial(r), r.steps)
        assert res[i].steps == r.steps and res[i].n == r.n
        np.testing.assert_array_equal(res[i].positions, ex)
        if ep is None:
            assert res[i].polarity is None
        else:
            np.testing.assert_array_equal(res[i].polarity, ep)


def check_snapshots(reqs, sink, every=10):
    want = {(i, s) for i, r in enumerate(reqs) for s in range(every, r.steps, every)}
    assert set(sink.got) == want
    for (i, s), (pos, pol) in sink.got.items():
        ex, ep = advanced(*initial(reqs[i]), s)
        np.testing.assert_array_equal(pos, ex)
        if ep is not None:
            np.testing.assert_array_equal(pol, ep)


def test_every_request_runs_its_steps_and_snapshots():
    reqs = stream(REQS)
    sink = Sink()
    srv, res = serve(reqs, sink=sink)
    check_results(reqs, res)
    check_snapshots(reqs, sink)
    assert srv.writer.written == len(sink.got) and not srv.writer.errors
    assert srv.cell_steps == sum(r.n * r.steps for r in reqs)
    eng = srv.lanes[0].engine
    assert all(k == 1 for k in eng.steps)
    assert all(slot_taken[1] % 10 == 0 for slot_taken in eng.snaps)


@pytest.mark.parametrize("k", [3, 8, 64])
def test_multi_step_issue_keeps_results_and_snapshot_steps(k):
    reqs = stream(REQS)
    sink = Sink()
    srv, res = serve(reqs, sink=sink, steps_per_issue=k)
    check_results(reqs, res)
    check_snapshots(reqs, sink)
    eng = srv.lanes[0].engine
    assert max(eng.steps) <= min(k, 10) and max(eng.steps) > 1
    # every request was downloaded after exactly its own step count
    assert sorted(t for _, t in eng.downloads) == sorted(r.steps for r in reqs)


def test_size_classes_route_each_request_to_its_lane():
    reqs = stream(REQS)
    sink = Sink()
    srv, res = serve(reqs, sink=sink, size_classes=[(500, 0.3), (None, 0.7)], steps_per_issue=4)
    check_results(reqs, res)
    check_snapshots(reqs, sink)
    small, large = (lane.engine for lane in srv.lanes)
    assert sorted(small.adds) == sorted(r.n for r in reqs if r.n <= 500)
    assert sorted(large.adds) == sorted(r.n for r in reqs if r.n > 500)
    assert (small.cells, large.cells) == (6_000, 14_000)


def test_size_classes_need_a_class_for_any_request():
    with pytest.raises(ValueError):
        HostServer(1000, 1000, size_classes=[(500, 0.5), (5000, 0.5)])


def test_admission_waits_for_free_cells_first_come_first_served():
    reqs = stream([(1500, 12), (1500, 12), (1500, 12), (400, 12)])
    srv, res = serve(reqs, cells=3_200)
    check_results(reqs, res)
    eng = srv.lanes[0].engine
    assert eng.peak_cells <= 3_200
    # the third request waits for the first two; the fourth, though it would fit, waits behind the third
    assert eng.adds == [1500, 1500, 1500, 400]
    adm = [res[i].admitted for i in range(4)]
    assert adm == sorted(adm)
    assert adm[2] >= min(res[0].completed, res[1].completed)


def test_request_larger_than_its_engine_is_refused_up_front():
    reqs = stream([(300, 5), (5000, 5)])
    with pytest.raises(ValueError, match="exceeds its engine"):
        serve(reqs, cells=4_000)


def test_resume_runs_only_the_remaining_steps():
    reqs = stream(REQS)
    sink = Sink()
    serve(reqs, sink=sink)
    # request 1 restarts from its step-30 snapshot, request 3 from step 10; request 2 (7 steps) is complete
    done2 = advanced(*initial(reqs[2]), 7)
    resume = {1: (30,) + sink.got[(1, 30)], 3: (10,) + sink.got[(3, 10)], 2: (7,) + done2}
    sink2 = Sink()
    srv, res = serve(reqs, sink=sink2, resume=resume, steps_per_issue=8)
    check_results(reqs, res)
    # resumed requests write only the snapshots after their resume step
    want = {(i, s) for i, r in enumerate(reqs) for s in range(10, r.steps, 10)
            if s > (resume[i][0] if i in resume else 0)}
    assert set(sink2.got) == want
    taken = sorted(t for _, t in srv.lanes[0].engine.downloads)
    assert taken == sorted(r.steps - (resume[i][0] if i in resume else 0) for i, r in enumerate(reqs))


def test_resume_state_must_match_the_request():
    reqs = stream(REQS[:2])
    x, p = initial(reqs[0])
    with pytest.raises(ValueError, match="does not match"):
        serve(reqs, resume={0: (5, x[:-1], p)})
    with pytest.raises(ValueError, match="does not match"):
        serve(reqs, resume={0: (reqs[0].steps + 1, x, p)})
    # polarity given for the spring request, or left out for the polarity one
    assert p is None
    with pytest.raises(ValueError, match="does not match"):
        serve(reqs, resume={0: (5, x, np.zeros((len(x), 2), np.float32))})
    x1, p1 = initial(reqs[1])
    assert p1 is not None
    with pytest.raises(ValueError, match="does not match"):
        serve(reqs, resume={1: (5, x1, None)})


def test_a_failing_sink_loses_only_that_snapshot():
    reqs = stream(REQS)
    sink = Sink(fail_at=(1, 20))
    srv, res = serve(reqs, sink=sink)
    check_results(reqs, res)
    assert (1, 20) not in sink.got and (1, 30) in sink.got
    assert srv.writer.errors == ["request 1 step 20: disk full"]


def test_resumed_server_continues_its_snapshot_files(tmp_path):
    """A server stops after step 25 of each request; a new one resumes them from their newest snapshots
    with an appending sink.  Each request's HDF5 file and XDMF sidecar end byte for byte as those of one
    uninterrupted run."""
    import dataclasses

    from tecs_gb300 import h5

    reqs = stream([(300, 47), (1200, 40), (150, 33)])
    one = h5.SnapshotSink(tmp_path / "one", dt=DT)
    serve(reqs, sink=one)
    one.close()
    first = h5.SnapshotSink(tmp_path / "two", dt=DT)
    serve([dataclasses.replace(r, steps=25) for r in reqs], sink=first)  # stops after step 25
    for w in first.files.values():
        w.f.close()  # left unclosed, as by a server that stopped
    resume = served.resume_points(tmp_path / "two", range(len(reqs)))
    assert {i: r[0] for i, r in resume.items()} == {0: 20, 1: 20, 2: 20}
    again = h5.SnapshotSink(tmp_path / "two", dt=DT, append=True)
    _, res = serve(reqs, sink=again, resume=resume, steps_per_issue=8)
    again.close()
    check_results(reqs, res)
    for i in range(len(reqs)):
        for ext in ("h5", "xmf"):
            name = f"request_{i:05d}.{ext}"
            assert (tmp_path / "two" / name).read_bytes() == (tmp_path / "one" / name).read_bytes(), name
