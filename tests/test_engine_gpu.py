"""The multi-simulation engine against plain single-simulation runs (GB300).

Every simulation the engine advances must evolve exactly as the plain
drop-in path (tecs_gb300.Simulation) evolves it: same pairs, same summation
order, so the trajectories are bit-identical -- for the spring laws with both
binned finders and both integrators.  Polarity simulations agree within the
parity tests' tolerance with plain runs (same device code, per-thread path).
Admission and retirement between steps must not disturb the others.
"""
import numpy as np
import pytest

import tecs_gb300 as tg
from tecs_gb300 import workloads as wl
from tecs_gb300.engine import Engine, bins_needed

pytestmark = pytest.mark.gpu


def spec(n, seed, finder, integrator, k_rep=2.0, k_adh=0.5, polarity=False):
    x = wl.ball(n, seed)
    mn, mx = wl.bounds_for(x)
    pf = tg.PairFinderSettings(min_bounds=mn, max_bounds=mx)
    force = tg.PolaritySpring(k_rep=k_rep, k_adh=k_adh) if polarity else tg.Spring2R(k_rep=k_rep, k_adh=k_adh)
    settings = tg.Settings(agent_count=n, capacity=n, pair_finder_settings=pf)
    d = tg.make_desc(settings, pair_finder=finder, integrator=integrator, force=force, polarity=polarity)
    p = wl.outward_polarity(x, seed) if polarity else None
    return x, p, d, settings, force


def plain_run(x, p, settings, finder, integrator, force, polarity, steps, dt=0.05):
    s = tg.Simulation(settings, pair_finder=finder, integrator=integrator, force=force, polarity=polarity)
    s.set_state(x, p)
    s.take_step(dt, steps)
    return s.get_state()


def test_engine_matches_plain_runs_bit_for_bit():
    cases = [(1500, 1, "binned_gabriel", "heun", 2.0, 0.5), (800, 2, "binned_all_pairs", "heun", 1.7, 0.4),
             (3000, 3, "binned_gabriel", "euler", 2.3, 0.6), (500, 4, "binned_all_pairs", "euler", 1.5, 0.3),
             (6000, 5, "binned_gabriel", "heun", 2.1, 0.7)]
    specs = [spec(n, sd, f, it, kr, ka) for n, sd, f, it, kr, ka in cases]
    eng = Engine(cell_capacity=20000, bin_capacity=sum(bins_needed(s[2]) for s in specs) + 1000, max_sims=16)
    slots = [eng.add(d, x, p) for x, p, d, _, _ in specs]
    eng.step(0.05, 6)
    for (x, p, d, settings, force), slot, case in zip(specs, slots, cases):
        xe, _ = eng.download(slot)
        xp, _ = plain_run(x, p, settings, case[2], case[3], force, False, 6)
        np.testing.assert_array_equal(xe, xp)


def test_engine_admission_and_retirement():
    a = spec(2000, 11, "binned_gabriel", "heun")
    b = spec(1200, 12, "binned_gabriel", "euler")
    c = spec(1700, 13, "binned_all_pairs", "heun")
    eng = Engine(cell_capacity=6000, bin_capacity=sum(bins_needed(s[2]) for s in (a, b, c)) + 100, max_sims=4)
    sa = eng.add(a[2], a[0])
    sb = eng.add(b[2], b[0])
    eng.step(0.05, 3)
    eng.remove(sb)
    sc = eng.add(c[2], c[0])
    eng.step(0.05, 4)
    assert eng.count() == (2000 + 1700, 2)
    xa, _ = eng.download(sa)
    np.testing.assert_array_equal(xa, plain_run(a[0], None, a[3], "binned_gabriel", "heun", a[4], False, 7)[0])
    xc, _ = eng.download(sc)
    np.testing.assert_array_equal(xc, plain_run(c[0], None, c[3], "binned_all_pairs", "heun", c[4], False, 4)[0])


def test_engine_polarity_close_to_plain():
    x = wl.sheet(2500, 21)
    p = wl.outward_polarity(x, 21)
    mn, mx = wl.bounds_for(x)
    settings = tg.Settings(agent_count=2500, capacity=2500, pair_finder_settings=tg.PairFinderSettings(
        min_bounds=mn, max_bounds=mx))
    force = tg.PolaritySpring(k_pol=0.2)
    d = tg.make_desc(settings, pair_finder="binned_gabriel", integrator="heun", force=force, polarity=True)
    other = spec(3000, 22, "binned_gabriel", "heun")
    eng = Engine(cell_capacity=8000, bin_capacity=bins_needed(d) + bins_needed(other[2]) + 10, max_sims=4)
    s1 = eng.add(d, x, p)
    eng.add(other[2], other[0])
    eng.step(0.05, 3)
    xe, pe = eng.download(s1)
    xp, pp = plain_run(x, p, settings, "binned_gabriel", "heun", force, True, 3)
    np.testing.assert_array_equal(xe, xp)
    np.testing.assert_array_equal(pe, pp)


def test_engine_snapshot_async_matches_download():
    import torch

    a = spec(4000, 31, "binned_gabriel", "heun")
    eng = Engine(cell_capacity=5000, bin_capacity=bins_needed(a[2]) + 10, max_sims=2)
    s = eng.add(a[2], a[0])
    eng.step(0.05, 2)
    host = torch.empty((4000, 3), dtype=torch.float32, pin_memory=True)
    ev = eng.snapshot_async(s, host.data_ptr(), None)
    eng.step(0.05, 1)  # the snapshot must hold the state before this step
    eng.synchronize()
    assert Engine.event_ready(ev)
    Engine.event_destroy(ev)
    ref = plain_run(a[0], None, a[3], "binned_gabriel", "heun", a[4], False, 2)[0]
    np.testing.assert_array_equal(host.numpy(), ref)


def test_engine_rejects_what_it_cannot_run():
    x, _, d, _, _ = spec(100, 41, "binned_gabriel", "heun")
    eng = Engine(cell_capacity=150, bin_capacity=2 * bins_needed(d) + 1, max_sims=2)
    d.com_fix = 1
    with pytest.raises(tg.TecsError):
        eng.add(d, x)
    d.com_fix = 0
    eng.add(d, x)
    with pytest.raises(tg.TecsError, match="capacity"):
        eng.add(d, x)


def test_idle_engine_returns_everything_at_remove():
    a = spec(3000, 51, "binned_gabriel", "heun")
    b = spec(2000, 52, "binned_all_pairs", "euler")
    nb = bins_needed(a[2]) + bins_needed(b[2])
    eng = Engine(cell_capacity=5000, bin_capacity=nb, max_sims=4)
    sa = eng.add(a[2], a[0])
    sb = eng.add(b[2], b[0])
    eng.step(0.05, 2)
    eng.remove(sa)
    assert eng.free()[0] == 0  # cells of a removed simulation leave at the next sort
    eng.remove(sb)
    assert eng.free() == (5000, nb)  # nothing active: all returned without a step
    sc = eng.add(a[2], a[0])
    eng.step(0.05, 3)
    xc, _ = eng.download(sc)
    np.testing.assert_array_equal(xc, plain_run(a[0], None, a[3], "binned_gabriel", "heun", a[4], False, 3)[0])


def test_engine_after_other_engines_closed_matches_plain_runs():
    # Engines created and closed first (as the bin-scale autotuner does) leave
    # freed device memory that a new engine may reuse: its clears must be
    # ordered before its first kernels, or stale contents leak into the step.
    from tecs_gb300 import batched

    members = batched.ensemble(24, 7, lo=500, hi=20_000)
    for scale in (1.0, 1.25, 1.5):
        eng, _ = batched.build_engine(members, {"small": scale, "medium": scale, "large": scale})
        eng.step(0.05, 2)
        eng.close()
    eng, slots = batched.build_engine(members, {})
    eng.step(0.05, 5)
    for m, slot in zip(members, slots):
        xe, _ = eng.download(slot)
        s = tg.Simulation(m.settings, pair_finder=m.finder, integrator=m.integrator, force=m.force)
        s.set_state(m.x)
        s.take_step(0.05, 5)
        np.testing.assert_array_equal(xe, s.get_state()[0])
        s.close()
    eng.close()


@pytest.mark.parametrize("threads", [64, 128])
def test_engine_block_size_changes_no_result(threads):
    """The force passes at 64 or 128 threads per block (the autotuner's other choices) give the plain runs'
    trajectories bit for bit, also with a polarity simulation resident; a change between steps recaptures
    the step graph."""
    cases = [(1500, 61, "binned_gabriel", "heun"), (900, 62, "binned_all_pairs", "euler"),
             (4000, 63, "binned_gabriel", "euler")]
    specs = [spec(n, sd, f, it) for n, sd, f, it in cases]
    pol = spec(1200, 64, "binned_gabriel", "heun", polarity=True)
    eng = Engine(cell_capacity=12000, bin_capacity=sum(bins_needed(s[2]) for s in specs + [pol]) + 100, max_sims=8)
    slots = [eng.add(d, x, p) for x, p, d, _, _ in specs]
    sp = eng.add(pol[2], pol[0], pol[1])
    eng.step(0.05, 2)
    eng.set_pass_threads(threads)
    eng.step(0.05, 3)
    for (x, p, d, settings, force), slot, case in zip(specs, slots, cases):
        xe, _ = eng.download(slot)
        np.testing.assert_array_equal(xe, plain_run(x, p, settings, case[2], case[3], force, False, 5)[0])
    xe, pe = eng.download(sp)
    xp, pp = plain_run(pol[0], pol[1], pol[3], "binned_gabriel", "heun", pol[4], True, 5)
    np.testing.assert_array_equal(xe, xp)
    np.testing.assert_array_equal(pe, pp)
    with pytest.raises(tg.TecsError, match="64, 96 or 128"):
        eng.set_pass_threads(100)
