"""One-cluster steps of small simulations (k_step_small) against the multi-kernel step (GB300).

A simulation of up to 1536 cells on a grid of up to 16384 bins (Euler, binned
finder on the cooperative pass's geometry, built-in law, no COM fix, no
division) takes its whole step in one launch of one cluster of blocks.  The
step must equal the multi-kernel one bit for bit: both binned finders, the
polarity law, 2-D, and rebuilds every step or every few steps; and
the bin counts it leaves behind must serve a later evaluate() exactly as the
multi-kernel step's do.  TECS_NO_SMALL_STEP=1 at creation selects the
multi-kernel step.
"""
import os

import numpy as np
import pytest

import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

CASES = [
    ("binned_all_pairs", "euler", 3, False, 0, 1000),
    ("binned_gabriel", "euler", 3, False, 0, 1500),
    ("binned_gabriel", "euler", 3, False, 0, 2000),  # past the limit: the grid path
    ("binned_gabriel", "euler", 3, True, 0, 1500),
    ("binned_all_pairs", "euler", 2, False, 0, 1000),
    ("binned_gabriel", "euler", 3, False, 3, 1200),
    ("binned_gabriel", "heun", 3, False, 0, 1000),  # Heun: the grid path
]


def make(finder, integrator, dims, pol, every, n, small):
    os.environ["TECS_NO_SMALL_STEP"] = "0" if small else "1"
    try:
        if pol:
            x = wl.sheet(n, 3)
            p = wl.outward_polarity(x, 3)
        else:
            x = wl.ball(n, 4, radius=(n / 4.19) ** (1 / 3))
            p = None
        if dims == 2:
            x = np.ascontiguousarray(x[:, :2])
        m = float(np.ceil(np.abs(x).max() + 2))
        pf = tg.PairFinderSettings(min_bounds=(-m,) * 3, max_bounds=(m,) * 3, rebuild_every_n=every)
        force = tg.PolaritySpring(k_pol=0.2) if pol else tg.Spring2R()
        s = tg.Simulation(tg.Settings(agent_count=n, capacity=n, cutoff_distance=1.0, pair_finder_settings=pf),
                          dims=dims, pair_finder=finder, integrator=integrator, force=force, polarity=pol)
        s.set_state(x, p)
        return s
    finally:
        os.environ.pop("TECS_NO_SMALL_STEP", None)


@pytest.mark.parametrize("finder,integrator,dims,pol,every,n", CASES)
def test_one_block_step_equals_the_multi_kernel_step(finder, integrator, dims, pol, every, n):
    a = make(finder, integrator, dims, pol, every, n, small=True)
    b = make(finder, integrator, dims, pol, every, n, small=False)
    a.take_step(0.05, 7)
    b.take_step(0.05, 7)
    xa, pa = a.get_state()
    xb, pb = b.get_state()
    np.testing.assert_array_equal(xa, xb)
    if pol:
        np.testing.assert_array_equal(pa, pb)
    # the counts a step leaves for the next rebuild serve evaluate() too
    da, _, qa = a.evaluate()
    db, _, qb = b.evaluate()
    np.testing.assert_array_equal(da, db)
    np.testing.assert_array_equal(tg.canonical_pairs(qa), tg.canonical_pairs(qb))
    a.take_step(0.05, 3)
    b.take_step(0.05, 3)
    np.testing.assert_array_equal(a.get_state()[0], b.get_state()[0])
    if every == 0 and n <= 1536 and integrator == "euler":
        assert a.kernels_per_step() == 1 and b.kernels_per_step() > 1
    elif every == 0:
        assert a.kernels_per_step() == b.kernels_per_step() > 1


def test_force_changed_after_creation_takes_the_one_launch_step():
    # tecs_sim_set_force picks another instantiation of the kernel than the
    # one the simulation was created with; each must be ready to launch
    L = tg.load()
    sims = [make("binned_all_pairs", "euler", 3, False, 0, 1000, small=f) for f in (True, False)]
    for s in sims:
        s.take_step(0.05, 2)
        tg._check(L.tecs_sim_set_force(s._h, 0, 0.0, 0.0, 0.0, 0.0, 0.0))  # no force
        s.take_step(0.05, 2)
        tg._check(L.tecs_sim_set_force(s._h, 1, 1.5, 0.6, 0.4, 0.9, 0.0))
        s.take_step(0.05, 3)
    np.testing.assert_array_equal(sims[0].get_state()[0], sims[1].get_state()[0])
    assert sims[0].kernels_per_step() == 1 and sims[1].kernels_per_step() > 1
