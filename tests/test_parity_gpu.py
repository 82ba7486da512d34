"""CUDA path vs the CPU oracle on the same seeded inputs (GB300).

Bars:
  * pair lists: canonical directed (self, other) id lists identical, bit for bit;
  * spring deltas and whole Euler / Heun runs without the COM fix: identical
    (the kernels keep the reference's summation order and contract no FMA);
  * with the COM fix, symmetric finders or the polarity law: per component
    |gpu - cpu| <= RTOL * |cpu| + ATOL * rms(cpu), RTOL = 1e-5, ATOL = 1e-6
    (sin/cos/acos/atan2 and the COM sum are not bit-reproducible across libm
    and CUDA; ATOL covers components that cancel to ~0).
"""
import numpy as np
import pytest

import oracle
import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

RTOL = 1e-5
ATOL = 1e-6

FINDER_MAP = {
    "naive_all_pairs": oracle.NAIVE_ALL_PAIRS,
    "binned_all_pairs": oracle.BINNED_ALL_PAIRS,
    "naive_gabriel": oracle.NAIVE_GABRIEL,
    "binned_gabriel": oracle.BINNED_GABRIEL,
    "naive_delaunay": oracle.NAIVE_DELAUNAY,
}


def close(gpu, cpu, rtol=RTOL, atol=ATOL):
    gpu = np.asarray(gpu, np.float64)
    cpu = np.asarray(cpu, np.float64)
    scale = np.sqrt(np.mean(cpu ** 2)) if cpu.size else 0.0
    err = np.abs(gpu - cpu)
    tol = rtol * np.abs(cpu) + atol * scale
    bad = err > tol
    return not bad.any(), float(err.max() if err.size else 0.0), int(bad.sum())


def make_pair(x, *, finder, dims=3, integrator="heun", com=False, symmetric=False, force="spring", pol=None,
              bounds=None, capacity=None, division=0.0, bin_size_scale=1.0, rebuild_every_n=0, cutoff=1.0,
              k_pol=0.2, gab=0.8, graph=True):
    n = len(x)
    cap = capacity or max(n, 1)
    if bounds is None:
        bounds = wl.bounds_for(x) if n else ((-5,) * 3, (5,) * 3)
    mn, mx = bounds
    pf = tg.PairFinderSettings(gabriel_coefficient=gab, min_bounds=mn, max_bounds=mx, bin_size_scale=bin_size_scale,
                               rebuild_every_n=rebuild_every_n)
    if force == "spring":
        f_gpu, f_cpu = tg.Spring2R(), oracle.FORCE_SPRING2R
    elif force == "polarity":
        f_gpu, f_cpu = tg.PolaritySpring(k_pol=k_pol), oracle.FORCE_POLARITY
    else:
        f_gpu, f_cpu = None, oracle.FORCE_NONE
    g = tg.Simulation(tg.Settings(agent_count=n, capacity=cap, cutoff_distance=cutoff, pair_finder_settings=pf),
                      dims=dims, pair_finder=finder, symmetric=symmetric, integrator=integrator,
                      com_fixer="global" if com else None, force=f_gpu, polarity=pol is not None,
                      division=tg.Division(probability=division), graph=graph)
    c = oracle.Oracle(dims=dims, finder=FINDER_MAP[finder], symmetric=symmetric, cutoff=cutoff, gabriel_coefficient=gab,
                      min_bounds=mn, max_bounds=mx, bin_size_scale=bin_size_scale, rebuild_every_n=rebuild_every_n,
                      integrator=tg.INTEGRATORS[integrator], com_fix=com, force=f_cpu, k_pol=k_pol,
                      has_polarity=pol is not None, capacity=cap, division_probability=division)
    g.set_state(x, pol)
    c.set_state(x, pol)
    return g, c


def ball(n, seed=0, radius=None):
    return wl.ball(n, seed, radius)


# ---------------------------------------------------------------------------
# pair lists and one-pass deltas

@pytest.mark.parametrize("finder", ["binned_all_pairs", "binned_gabriel", "naive_all_pairs", "naive_gabriel"])
@pytest.mark.parametrize("dims", [3, 2])
def test_pairs_and_deltas_bit_exact(finder, dims):
    n = 1500 if finder.startswith("naive") else 4000
    x = ball(n, seed=11)
    if dims == 2:
        x = np.ascontiguousarray(x[:, :2] * 0.6)
    g, c = make_pair(x, finder=finder, dims=dims)
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    assert len(pc) > n  # non-trivial
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)


def test_binned_equals_naive_pair_set():
    x = ball(1200, seed=5)
    g1, _ = make_pair(x, finder="binned_gabriel")
    g2, _ = make_pair(x, finder="naive_gabriel")
    np.testing.assert_array_equal(tg.canonical_pairs(g1.evaluate()[2]), tg.canonical_pairs(g2.evaluate()[2]))


@pytest.mark.parametrize("finder", ["binned_all_pairs", "binned_gabriel", "naive_gabriel", "naive_all_pairs"])
def test_symmetric_pairs_exact_deltas_close(finder):
    n = 1200 if finder.startswith("naive") else 3000
    x = ball(n, seed=3)
    g, c = make_pair(x, finder=finder, symmetric=True)
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    ok, err, nbad = close(dg, dc)
    assert ok, (err, nbad)


def test_naive_all_pairs_symmetric_matches_reference_fixture():
    # naive_all_pairs_symmetric.hpp:82-155 run by the reference's own code
    # (tests/golden/make_golden.py, scenario nas_heun): j < i pairs, +delta to
    # i and -delta to j; float atomics here, so deltas and steps within tolerance
    from pathlib import Path
    gold = dict(np.load(Path(__file__).resolve().parent / "golden" / "nas_heun.npz"))
    prm = gold["prm"]
    x = gold["x0"]
    pf = tg.PairFinderSettings(min_bounds=tuple(prm[2:5]), max_bounds=tuple(prm[5:8]))
    s = tg.Simulation(tg.Settings(agent_count=len(x), capacity=len(x), cutoff_distance=float(prm[0]),
                                  pair_finder_settings=pf), pair_finder="naive_all_pairs", symmetric=True,
                      integrator="heun", force=tg.Spring2R())
    s.set_state(x)
    dg, _, pg = s.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(gold["pairs"]))
    ok, err, nbad = close(dg, gold["dpos"])
    assert ok, (err, nbad)
    s.take_step(float(gold["dt"]), int(gold["steps"]))
    ok, err, nbad = close(s.get_state()[0], gold["pos"])
    assert ok, (err, nbad)


def test_polarity_deltas_close():
    n = 3000
    x = wl.sheet(n, seed=4)
    p = wl.outward_polarity(x, seed=4)
    g, c = make_pair(x, finder="binned_gabriel", force="polarity", pol=p)
    dg, pg_, pairs_g = g.evaluate()
    dc, pc_, pairs_c = c.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pairs_g), tg.canonical_pairs(pairs_c))
    ok, err, nbad = close(dg, dc)
    assert ok, ("position deltas", err, nbad)
    ok, err, nbad = close(pg_, pc_)
    assert ok, ("polarity deltas", err, nbad)


# ---------------------------------------------------------------------------
# whole steps

def test_euler_binned_all_pairs_run_bit_exact():
    # small plain configuration: 1000 cells, ball R=5 (seed 0), rc 1.0, Euler dt 0.1
    x = wl.ball(1000, 0, radius=5.0)
    g, c = make_pair(x, finder="binned_all_pairs", integrator="euler", bounds=((-6,) * 3, (6,) * 3))
    g.take_step(0.1, 200)
    c.step(0.1, 200)
    xg, _ = g.get_state()
    xc, _ = c.get_state()
    np.testing.assert_array_equal(xg, xc)


@pytest.mark.parametrize("graph", [True, False])
def test_heun_gabriel_run_bit_exact(graph):
    x = ball(5000, seed=1)
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun", graph=graph)
    g.take_step(0.05, 20)
    c.step(0.05, 20)
    np.testing.assert_array_equal(g.get_state()[0], c.get_state()[0])


def test_heun_rebuild_every_n_stale_bins():
    x = ball(3000, seed=8)
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun", rebuild_every_n=4)
    g.take_step(0.05, 10)
    c.step(0.05, 10)
    np.testing.assert_array_equal(g.get_state()[0], c.get_state()[0])


def test_heun_com_close():
    x = ball(20000, seed=1)
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun", com=True, capacity=21000)
    g.take_step(0.05, 5)
    c.step(0.05, 5)
    ok, err, nbad = close(g.get_state()[0], c.get_state()[0])
    assert ok, (err, nbad)


def test_euler_com_symmetric_close():
    x = ball(3000, seed=2)
    g, c = make_pair(x, finder="binned_all_pairs", integrator="euler", com=True, symmetric=True)
    g.take_step(0.05, 5)
    c.step(0.05, 5)
    ok, err, nbad = close(g.get_state()[0], c.get_state()[0])
    assert ok, (err, nbad)


def test_polarity_heun_close():
    x = wl.sheet(4000, seed=6)
    p = wl.outward_polarity(x, seed=6)
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun", force="polarity", pol=p)
    g.take_step(0.05, 3)
    c.step(0.05, 3)
    xg, pg = g.get_state()
    xc, pc = c.get_state()
    ok, err, nbad = close(xg, xc, rtol=1e-5, atol=1e-5)
    assert ok, ("positions", err, nbad)
    ok, err, nbad = close(pg, pc, rtol=1e-5, atol=1e-5)
    assert ok, ("polarities", err, nbad)


def test_division_counts_and_positions():
    x = ball(20000, seed=9)
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun", com=True, capacity=24000, division=2e-3)
    g.take_step(0.05, 4)
    c.step(0.05, 4)
    assert g.get_agent_count() == c.count > 20000
    ok, err, nbad = close(g.get_state()[0], c.get_state()[0], atol=1e-5)
    assert ok, (err, nbad)


# ---------------------------------------------------------------------------
# edge cases the reference's pair finders meet

def test_empty_and_single_cell():
    for n in (0, 1):
        x = np.zeros((n, 3), np.float32)
        g, c = make_pair(x, finder="binned_gabriel", bounds=((-5,) * 3, (5,) * 3), capacity=4)
        g.take_step(0.05, 2)
        c.step(0.05, 2)
        assert g.get_agent_count() == n
        np.testing.assert_array_equal(g.get_state()[0], c.get_state()[0])


def test_cells_outside_bounds_clamped_and_crowded_bins():
    # the default +-20 grid with a domain that leaves it: edge bins get crowded
    x = ball(2000, seed=12, radius=26.0)
    g, c = make_pair(x, finder="binned_gabriel", bounds=((-20,) * 3, (20,) * 3), bin_size_scale=1.0)
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)


def test_dense_cluster_large_bins():
    # > 24 cells per bin exercises the in-place sort path
    x = ball(3000, seed=13, radius=2.5)
    g, c = make_pair(x, finder="binned_all_pairs", bin_size_scale=2.0, bounds=((-3,) * 3, (3,) * 3))
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    ok, err, nbad = close(dg, dc)
    assert ok


def test_coincident_cells():
    x = ball(500, seed=14)
    x[10] = x[11]
    g, c = make_pair(x, finder="binned_all_pairs")
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)


def test_rerun_bit_identical():
    x = ball(20000, seed=15)
    runs = []
    for _ in range(2):
        g, _ = make_pair(x, finder="binned_gabriel", com=True, division=1e-3, capacity=22000)
        g.take_step(0.05, 5)
        runs.append(g.get_state()[0])
    np.testing.assert_array_equal(runs[0], runs[1])


def test_full_size_million_cells_pairs_and_deltas():
    # the headline spheroid (1,000,000 cells, density 1, seed 1): one full-step
    # Gabriel + spring evaluation compared pair for pair and bit for bit
    x = wl.ball(1_000_000, 1)
    g, c = make_pair(x, finder="binned_gabriel", com=True, capacity=1_050_000)
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate(threads=0)
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)


@pytest.mark.parametrize("gab", [0.95, 1.0, 0.5])
def test_gabriel_coefficients_general_path(gab):
    # c > 0.9 takes the reference-shaped general path; c = 0.5 the fast paths
    x = ball(4000, seed=16)
    g, c = make_pair(x, finder="binned_gabriel", gab=gab)
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)


def test_dense_packing_neighbour_overflow():
    # ~3x the headline density: many cells exceed the 16-neighbour fast-path list
    x = ball(6000, seed=17, radius=8.0)
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun")
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)
    g.take_step(0.05, 3)
    c.step(0.05, 3)
    np.testing.assert_array_equal(g.get_state()[0], c.get_state()[0])


# ---------------------------------------------------------------------------
# naive Delaunay (naive_delaunay.hpp): a pair is applied once per accepted
# simplex, so pair lists are compared as multisets and sums stay in j order

@pytest.mark.parametrize("dims,n,integrator,steps", [(2, 300, "euler", 4), (3, 90, "heun", 2)])
def test_delaunay_pairs_deltas_and_steps_bit_exact(dims, n, integrator, steps):
    x = ball(n, seed=21)
    if dims == 2:
        x = np.ascontiguousarray(x[:, :2])
    bounds = ((-20,) * 3, (20,) * 3)
    g, c = make_pair(x, finder="naive_delaunay", dims=dims, integrator=integrator, bounds=bounds)
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    assert len(np.unique(pc, axis=0)) < len(pc)  # some pairs apply more than once
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)
    g.take_step(0.02, steps)
    c.step(0.02, steps)
    np.testing.assert_array_equal(g.get_state()[0], c.get_state()[0])


@pytest.mark.parametrize("name", ["nd_euler_2d", "nd_euler_2d_points11", "nd_heun_3d"])
def test_delaunay_matches_reference_fixtures(name):
    # the fixtures hold the reference's own outputs (tests/golden/make_golden.py)
    from pathlib import Path
    gold = dict(np.load(Path(__file__).resolve().parent / "golden" / f"{name}.npz"))
    prm = gold["prm"]
    dims = gold["x0"].shape[1]
    x = gold["x0"]
    pf = tg.PairFinderSettings(min_bounds=tuple(prm[2:5]), max_bounds=tuple(prm[5:8]))
    integ = "heun" if name.endswith("3d") else "euler"
    s = tg.Simulation(tg.Settings(agent_count=len(x), capacity=len(x), cutoff_distance=float(prm[0]),
                                  pair_finder_settings=pf), dims=dims, pair_finder="naive_delaunay",
                      integrator=integ, force=tg.Spring2R())
    s.set_state(x)
    dg, _, pg = s.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(gold["pairs"]))
    np.testing.assert_array_equal(dg, gold["dpos"])
    s.take_step(float(gold["dt"]), int(gold["steps"]))
    np.testing.assert_array_equal(s.get_state()[0], gold["pos"])


def test_delaunay_rejects_symmetric_and_large_capacity():
    x = ball(50, seed=2)
    with pytest.raises(tg.TecsError):
        make_pair(x, finder="naive_delaunay", symmetric=True)
    with pytest.raises(tg.TecsError, match="4096"):
        make_pair(x, finder="naive_delaunay", capacity=5000)


def test_delaunay_edge_cases():
    # two cells: no third point, no simplex, no pair; collinear 2-D points:
    # every circumcircle is degenerate (|den| <= eps), so no pair either
    for x in (np.array([[0, 0, 0], [0.5, 0, 0]], np.float32),
              np.array([[0, 0], [0.3, 0], [0.6, 0], [0.9, 0]], np.float32)):
        dims = x.shape[1]
        g, c = make_pair(x, finder="naive_delaunay", dims=dims, integrator="euler", bounds=((-5,) * 3, (5,) * 3))
        dg, _, pg = g.evaluate()
        dc, _, pc = c.evaluate()
        assert len(pg) == len(pc) == 0
        np.testing.assert_array_equal(dg, dc)
    # a square's four cocircular corners: whether the fourth corner counts as
    # inside a circumcircle (<= r^2) is decided by rounding, and the directed
    # pair list comes out asymmetric; the CUDA path must round as the oracle does
    x = np.array([[0, 0], [0.7, 0], [0.7, 0.7], [0, 0.7]], np.float32)
    g, c = make_pair(x, finder="naive_delaunay", dims=2, integrator="euler", bounds=((-5,) * 3, (5,) * 3))
    np.testing.assert_array_equal(tg.canonical_pairs(g.evaluate()[2]), tg.canonical_pairs(c.evaluate()[2]))


def test_huge_sparse_grid_scan():
    # a +-300 grid (216M bins, ~53k scan chunks in 13 super-chunk sums) around a
    # small ball: the bin scan must stay exact where the chunk partials are
    # summed in two levels
    x = ball(3000, seed=31)
    g, c = make_pair(x, finder="binned_gabriel", bounds=((-300,) * 3, (300,) * 3))
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate()
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)
    g.take_step(0.05, 2)
    c.step(0.05, 2)
    np.testing.assert_array_equal(g.get_state()[0], c.get_state()[0])
