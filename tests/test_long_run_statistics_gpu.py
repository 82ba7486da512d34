"""Long runs compared by trajectory statistics (GB300 vs the oracle).

Where the per-step results agree only to rounding (the polarity law's
transcendentals, the centre-of-mass sum, division), long trajectories are
compared by statistics rather than cell by cell:

  * mean in-cutoff neighbour count   |gpu - cpu| <= 1e-3 * cpu
  * radius of gyration               |gpu - cpu| <= 1e-4 * cpu
  * polarity order parameter |sum p_hat| / N (polarity runs)   |gpu - cpu| <= 1e-3

sampled along the run; the agent count after division must be exact (the
division decisions are integer hash comparisons on both sides).  The
tolerances are stated for runs of a few hundred steps, where the rounding
differences have had time to grow but not to change the tissue's state.
"""
import numpy as np
import pytest
from scipy.spatial import cKDTree

import oracle
import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def mean_neighbours(x, rc=1.0):
    t = cKDTree(x.astype(np.float64))
    return float(np.mean([len(v) - 1 for v in t.query_ball_point(x.astype(np.float64), rc * (1 - 1e-6))]))


def radius_of_gyration(x):
    x = x.astype(np.float64)
    return float(np.sqrt(((x - x.mean(0)) ** 2).sum(1).mean()))


def polarity_order(p):
    th, ph = p[:, 0].astype(np.float64), p[:, 1].astype(np.float64)
    v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
    return float(np.linalg.norm(v.sum(0)) / len(v))


def pair(x, p, *, com, division, force, capacity):
    mn, mx = wl.bounds_for(x)
    pol = p is not None
    g = tg.Simulation(tg.Settings(agent_count=len(x), capacity=capacity, pair_finder_settings=tg.PairFinderSettings(
        min_bounds=mn, max_bounds=mx)), pair_finder="binned_gabriel", integrator="heun",
        com_fixer="global" if com else None, force=force, polarity=pol, division=tg.Division(probability=division))
    c = oracle.Oracle(finder=oracle.BINNED_GABRIEL, integrator=oracle.HEUN, com_fix=com, min_bounds=mn, max_bounds=mx,
                      capacity=capacity, force=oracle.FORCE_POLARITY if pol else oracle.FORCE_SPRING2R,
                      k_pol=0.2 if pol else 0.0, has_polarity=pol, division_probability=division)
    g.set_state(x, p)
    c.set_state(x, p)
    return g, c


def compare(g, c, chunks, steps_per_chunk, pol):
    for _ in range(chunks):
        g.take_step(0.05, steps_per_chunk)
        c.step(0.05, steps_per_chunk, 0)
        xg, pg = g.get_state()
        xc, pc = c.get_state()
        assert len(xg) == len(xc)
        ng, nc = mean_neighbours(xg), mean_neighbours(xc)
        assert abs(ng - nc) <= 1e-3 * nc, (ng, nc)
        rg, rc_ = radius_of_gyration(xg), radius_of_gyration(xc)
        assert abs(rg - rc_) <= 1e-4 * rc_, (rg, rc_)
        if pol:
            og, oc = polarity_order(pg), polarity_order(pc)
            assert abs(og - oc) <= 1e-3, (og, oc)


def test_spheroid_with_com_and_division_statistics():
    # the headline configuration at 20k cells: Gabriel, spring, Heun, COM every step, division 1e-3
    x = wl.ball(20_000, 1)
    g, c = pair(x, None, com=True, division=1e-3, force=tg.Spring2R(), capacity=26_000)
    compare(g, c, chunks=4, steps_per_chunk=50, pol=False)


def test_polarity_sheet_statistics():
    # the epithelial sheet at 5k cells: Gabriel, spring + 0.2 (bending + alignment), Heun
    x = wl.sheet(5_000, 2)
    p = wl.outward_polarity(x, 2)
    g, c = pair(x, p, com=False, division=0.0, force=tg.PolaritySpring(k_pol=0.2), capacity=5_000)
    compare(g, c, chunks=4, steps_per_chunk=50, pol=True)
