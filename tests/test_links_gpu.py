"""Link forces on the GB300 against the reference and the oracle (GB300).

The law is the constant pull of the reference's intercalation/sorting
examples (examples/intercalation.cpp:65-71), evaluated after the pairwise
forces and in link order (integrators/base.hpp:197-234).  Without the COM fix
the runs are bit-identical to the reference's own outputs
(tests/golden/lk_*.npz) and to the oracle; with it they agree within the COM
tolerance |gpu - ref| <= 1e-5 |ref| + 1e-6 rms(ref).
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def close(a, b, rtol=1e-5, atol=1e-6):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = np.sqrt(np.mean(b ** 2))
    return bool((np.abs(a - b) <= rtol * np.abs(b) + atol * scale).all())


@pytest.mark.parametrize("name,finder,integrator,com,exact", [
    ("lk_bg_heun", "binned_gabriel", "heun", False, True),
    ("lk_ba_euler_com", "binned_all_pairs", "euler", True, False),
])
def test_links_reproduce_reference(name, finder, integrator, com, exact):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    prm = g["prm"]
    n = len(g["x0"])
    cap = max(int(prm[13]), n)
    pf = tg.PairFinderSettings(min_bounds=tuple(prm[2:5]), max_bounds=tuple(prm[5:8]))
    s = tg.Simulation(tg.Settings(agent_count=n, capacity=cap, cutoff_distance=float(prm[0]), pair_finder_settings=pf),
                      pair_finder=finder, integrator=integrator, com_fixer="global" if com else None,
                      force=tg.Spring2R(k_rep=float(prm[8]), r_rep=float(prm[9]), k_adh=float(prm[10]),
                                        r_adh=float(prm[11])))
    s.set_state(g["x0"])
    s.set_links(g["links"], float(prm[15]))
    s.take_step(float(g["dt"]), int(g["steps"]))
    x, _ = s.get_state()
    if exact:
        np.testing.assert_array_equal(x, g["pos"])
    else:
        assert close(x, g["pos"])


@pytest.mark.parametrize("finder", ["binned_gabriel", "naive_all_pairs"])
def test_links_match_oracle_with_rebuild_every_n(finder):
    x = wl.ball(1500, 23)
    rng = np.random.default_rng(5)
    links = rng.integers(0, 1500, size=(600, 2)).astype(np.uint32)
    links[:20, 1] = links[:20, 0]  # self links are skipped
    mn, mx = wl.bounds_for(x)
    pf = tg.PairFinderSettings(min_bounds=mn, max_bounds=mx, rebuild_every_n=3)
    s = tg.Simulation(tg.Settings(agent_count=1500, capacity=1500, pair_finder_settings=pf), pair_finder=finder,
                      integrator="heun", force=tg.Spring2R())
    o = oracle.Oracle(finder=oracle.BINNED_GABRIEL if finder == "binned_gabriel" else oracle.NAIVE_ALL_PAIRS,
                      integrator=oracle.HEUN, min_bounds=mn, max_bounds=mx, rebuild_every_n=3, capacity=1500)
    s.set_state(x)
    o.set_state(x)
    s.set_links(links, 0.3)
    o.set_links(links, 0.3)
    s.take_step(0.05, 7)
    o.step(0.05, 7)
    np.testing.assert_array_equal(s.get_state()[0], o.get_state()[0])
    # removing the links restores the plain law; changing them does not
    # change the finder's rebuild schedule
    s.set_links(np.zeros((0, 2), np.uint32), 0.0)
    o.set_links(np.zeros((0, 2), np.uint32), 0.0)
    s.take_step(0.05, 3)
    o.step(0.05, 3)
    np.testing.assert_array_equal(s.get_state()[0], o.get_state()[0])
    # new links between rebuilds (the id -> slot map comes from the last sort)
    s.take_step(0.05, 1)
    o.step(0.05, 1)
    s.set_links(links[::-1], 0.4)
    o.set_links(links[::-1], 0.4)
    s.take_step(0.05, 5)
    o.step(0.05, 5)
    np.testing.assert_array_equal(s.get_state()[0], o.get_state()[0])


def test_links_with_division_and_com_close():
    x = wl.ball(3000, 29)
    rng = np.random.default_rng(9)
    links = rng.integers(0, 3000, size=(900, 2)).astype(np.uint32)
    mn, mx = wl.bounds_for(x)
    pf = tg.PairFinderSettings(min_bounds=mn, max_bounds=mx)
    s = tg.Simulation(tg.Settings(agent_count=3000, capacity=3400, pair_finder_settings=pf),
                      pair_finder="binned_gabriel", integrator="heun", com_fixer="global", force=tg.Spring2R(),
                      division=tg.Division(probability=2e-3))
    o = oracle.Oracle(finder=oracle.BINNED_GABRIEL, integrator=oracle.HEUN, com_fix=True, min_bounds=mn, max_bounds=mx,
                      capacity=3400, division_probability=2e-3)
    s.set_state(x)
    o.set_state(x)
    s.set_links(links, 0.25)
    o.set_links(links, 0.25)
    s.take_step(0.05, 10)
    o.step(0.05, 10)
    xg, _ = s.get_state()
    xc, _ = o.get_state()
    assert len(xg) == len(xc) > 3000
    assert close(xg, xc)


def test_link_validation():
    x = wl.ball(100, 3)
    s = tg.Simulation(tg.Settings(agent_count=100, capacity=100), pair_finder="binned_gabriel", force=tg.Spring2R())
    s.set_state(x)
    with pytest.raises(tg.TecsError, match="capacity"):
        s.set_links(np.array([[0, 100]], np.uint32), 0.1)
    sym = tg.Simulation(tg.Settings(agent_count=100, capacity=100), pair_finder="binned_gabriel", symmetric=True,
                        force=tg.Spring2R())
    with pytest.raises(tg.TecsError, match="non-symmetric"):
        sym.set_links(np.array([[0, 1]], np.uint32), 0.1)
