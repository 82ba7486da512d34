"""The served loop: continuous batching over the engine (GB300).

Requests arriving while others run are admitted at the next step and share
its launches; each request's result must equal the same simulation run alone
(the plain drop-in path) -- bit for bit, since the per-cell arithmetic and
summation order do not depend on what else is resident.  Snapshots stream to
HDF5 files through pinned buffers on a side stream.
"""
import numpy as np
import pytest

import tecs_gb300 as tg
from tecs_gb300 import h5
from tecs_gb300 import workloads as wl
from tecs_gb300.served import NativeServer, Server, request_sim, summarize

pytestmark = pytest.mark.gpu


def alone(req, max_cells, steps=None):
    x, p, d, settings, force = request_sim(req, max_cells)
    s = tg.Simulation(settings, pair_finder="binned_gabriel", integrator=req.integrator, force=force,
                      polarity=p is not None)
    s.set_state(x, p)
    s.take_step(0.05, req.steps if steps is None else steps)
    return s.get_state()


def test_results_same_alone_and_in_the_mix(tmp_path):
    reqs = wl.served_stream(14, seed=5, rate_hz=200.0, lo=800, hi=12000, steps_lo=20, steps_hi=130)
    sink = h5.SnapshotSink(tmp_path)
    # capacity for about three requests at a time: admissions wait for retirements
    srv = Server(cell_capacity=30000, bin_capacity=160000, max_sims=16, snapshot_every=50, sink=sink,
                 keep_results=True)
    res = srv.run(reqs, time_scale=1.0)
    srv.close()
    sink.close()
    assert len(res) == len(reqs)
    assert max(r.admitted for r in res) > min(r.completed for r in res)  # some admitted while others ran
    for r in res:
        x_alone, p_alone = alone(reqs[r.index], None)
        np.testing.assert_array_equal(r.positions, x_alone)
        if p_alone is not None:
            np.testing.assert_array_equal(r.polarity, p_alone)
    # snapshots: one group per 50 steps before the last, with the right shapes
    assert not srv.writer.errors
    for r in res:
        want = [f"t{k}" for k in range(50, reqs[r.index].steps, 50)]
        if not want:
            continue
        f = h5.H5File(tmp_path / f"request_{r.index:05d}.h5")
        assert sorted(f.keys()) == sorted(want)
        assert f.read(f"{want[0]}/position").shape == (reqs[r.index].n, 3)
    s = summarize(res, srv.makespan, srv.cell_steps)
    assert s["p99_s"] >= s["p50_s"] > 0


def test_failing_snapshot_sink_fails_only_that_snapshot(tmp_path):
    reqs = wl.served_stream(4, seed=6, rate_hz=1000.0, lo=1000, hi=3000, steps_lo=60, steps_hi=60)

    def sink(request, step, pos, pol):
        if request == 1:
            raise OSError(28, "No space left on device")

    srv = Server(cell_capacity=20000, bin_capacity=100000, max_sims=8, snapshot_every=25, sink=sink)
    res = srv.run(reqs)
    srv.close()
    assert len(res) == 4
    assert srv.writer.errors and all("request 1" in e for e in srv.writer.errors)


def test_size_classes_and_batched_issue_keep_results_and_snapshots(tmp_path):
    # two lanes: requests up to 3000 cells in one engine, the rest in another, each on its own stream
    reqs = wl.served_stream(12, seed=7, rate_hz=400.0, lo=800, hi=12000, steps_lo=30, steps_hi=150)
    # and up to 8 steps per engine call, never past a request's next snapshot or end
    sink = h5.SnapshotSink(tmp_path)
    srv = Server(cell_capacity=60000, bin_capacity=400000, max_sims=16, snapshot_every=40, sink=sink,
                 keep_results=True, size_classes=[(3000, 0.3), (None, 0.7)], steps_per_issue=8)
    res = srv.run(reqs, time_scale=1.0)
    srv.close()
    sink.close()
    assert len(res) == len(reqs)
    assert {r.n <= 3000 for r in res} == {True, False}  # both lanes served requests
    for r in res:
        x_alone, p_alone = alone(reqs[r.index], None)
        np.testing.assert_array_equal(r.positions, x_alone)
        if p_alone is not None:
            np.testing.assert_array_equal(r.polarity, p_alone)
    assert not srv.writer.errors
    for r in res:
        want = [f"t{k}" for k in range(40, reqs[r.index].steps, 40)]
        if want:
            assert sorted(h5.H5File(tmp_path / f"request_{r.index:05d}.h5").keys()) == sorted(want)


def test_size_classes_need_a_lane_for_any_request():
    with pytest.raises(ValueError):
        Server(cell_capacity=1000, bin_capacity=1000, size_classes=[(500, 1.0)])


def test_resume_from_snapshots_gives_the_uninterrupted_results(tmp_path):
    from tecs_gb300 import h5
    from tecs_gb300.served import resume_points

    reqs = wl.served_stream(6, seed=8, rate_hz=500.0, lo=800, hi=6000, steps_lo=90, steps_hi=140)
    sink = h5.SnapshotSink(tmp_path)
    srv = Server(cell_capacity=40000, bin_capacity=300000, max_sims=8, snapshot_every=40, sink=sink,
                 keep_results=True)
    full = {r.index: r for r in srv.run(reqs)}
    srv.close()
    sink.close()
    # resume every request from its newest snapshot (step 40 or 80) in a fresh server
    points = resume_points(tmp_path, range(len(reqs)))
    assert set(points) == set(range(len(reqs))) and {s for s, _, _ in points.values()} <= {40, 80, 120}
    srv2 = Server(cell_capacity=40000, bin_capacity=300000, max_sims=8, snapshot_every=40, sink=None,
                  keep_results=True, size_classes=[(3000, 0.4), (None, 0.6)], steps_per_issue=8)
    resumed = srv2.run(reqs, resume=points)
    srv2.close()
    assert len(resumed) == len(reqs)
    assert srv2.cell_steps == sum(r.n * (r.steps - points[r.index][0]) for r in resumed)
    for r in resumed:
        np.testing.assert_array_equal(r.positions, full[r.index].positions)
        if full[r.index].polarity is not None:
            np.testing.assert_array_equal(r.polarity, full[r.index].polarity)


@pytest.mark.parametrize("lanes,per_issue", [(None, 1), ([(3000, 0.3), (None, 0.7)], 8)])
def test_native_server_results_and_snapshots(tmp_path, lanes, per_issue):
    """The library's own served loop (tecs_serve_*: server and writer threads in C++): every request's result
    equals the same simulation run alone, bit for bit, with one lane or two size-class lanes and multi-step
    issue; the writer's HDF5 files hold one group per snapshot step, and a snapshot equals the plain run
    stopped at that step."""
    reqs = wl.served_stream(12, seed=9, rate_hz=300.0, lo=800, hi=12000, steps_lo=30, steps_hi=140)
    srv = NativeServer(cell_capacity=40000, bin_capacity=240000, max_sims=16, snapshot_every=40,
                       snapshot_dir=tmp_path, keep_results=True, size_classes=lanes, steps_per_issue=per_issue)
    res = srv.run(reqs, time_scale=1.0)
    srv.close()  # joins the writer: every file is closed
    assert len(res) == len(reqs) and srv.written > 0
    assert max(r.admitted for r in res) > min(r.completed for r in res)  # some admitted while others ran
    for r in res:
        req = reqs[r.index]
        x_alone, p_alone = alone(req, None)
        np.testing.assert_array_equal(r.positions, x_alone)
        if p_alone is not None:
            np.testing.assert_array_equal(r.polarity, p_alone)
        want = [f"t{k}" for k in range(40, req.steps, 40)]
        if not want:
            continue
        f = h5.H5File(tmp_path / f"request_{r.index:05d}.h5")
        assert sorted(f.keys(), key=lambda g: int(g[1:])) == want
        xs, ps = alone(req, None, steps=40)
        np.testing.assert_array_equal(f.read("t40/position"), xs)
        if ps is not None:
            np.testing.assert_array_equal(f.read("t40/polarity"), ps)
    s = summarize(res, srv.makespan, srv.cell_steps)
    assert s["p99_s"] >= s["p50_s"] > 0


def test_native_server_resume_ends_as_uninterrupted(tmp_path):
    """A request submitted with a start step (the state of its snapshot at that step) runs only its
    remaining steps and ends with the uninterrupted result."""
    reqs = wl.served_stream(3, seed=10, rate_hz=1000.0, lo=2000, hi=6000, steps_lo=90, steps_hi=90)
    (tmp_path / "a").mkdir()
    srv = NativeServer(cell_capacity=30000, bin_capacity=200000, max_sims=8, snapshot_every=30,
                       snapshot_dir=tmp_path / "a", keep_results=True)
    full = srv.run(reqs)
    srv.close()
    resume = {}
    for r in full:
        f = h5.H5File(tmp_path / "a" / f"request_{r.index:05d}.h5")
        pol = f.read("t60/polarity") if "polarity" in f.keys("t60") else None
        resume[r.index] = (60, f.read("t60/position"), pol)
    (tmp_path / "b").mkdir()
    srv = NativeServer(cell_capacity=30000, bin_capacity=200000, max_sims=8, snapshot_every=30,
                       snapshot_dir=tmp_path / "b", keep_results=True)
    again = srv.run(reqs, resume=resume)
    srv.close()
    for a, b in zip(full, again):
        np.testing.assert_array_equal(a.positions, b.positions)
        if a.polarity is not None:
            np.testing.assert_array_equal(a.polarity, b.polarity)
