"""The standalone bin grid (tecs_grid_*) against the reference's acceleration::Grid.

The fixtures grid_q_3d / grid_q_2d hold the reference's own query results
(include/utils/grid.hpp:413-637, run by tests/golden/make_golden.py): nearest
point in 3^d and 5^d bins, a random point of the 3^d bins, a random point
within a physical radius, and the same among indices not divisible by 3, the
random targets fixed by recorded draws.  Indices are compared exactly; a
larger seeded case is compared with the oracle's restatement.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle
import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def run_all(grid, q, draws, radius, n):
    eligible = (np.arange(n) % 3 != 0).astype(np.uint8)
    return {"near1": grid.nearest(q, 1), "near2": grid.nearest(q, 2), "rbins": grid.random_in_bins(q, 1, draws),
            "rrad": grid.random_in_radius(q, radius, draws),
            "rfilt": grid.random_in_radius(q, radius, draws, eligible=eligible)}


@pytest.mark.parametrize("name", ["grid_q_3d", "grid_q_2d"])
def test_grid_queries_match_reference(name):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    prm = g["prm"]
    dims = g["x"].shape[1]
    grid = tg.Grid(dims, prm[2:2 + dims], prm[5:5 + dims], float(prm[0]), len(g["x"]))
    grid.rebuild(g["x"])
    out = run_all(grid, g["q"], g["draws"], float(prm[1]), len(g["x"]))
    for k, v in out.items():
        np.testing.assert_array_equal(v, g[k], err_msg=k)
    # a rebuild over other points replaces the first
    grid.rebuild(g["x"][::2])
    np.testing.assert_array_equal(grid.nearest(g["q"], 1),
                                  oracle.grid_query(g["x"][::2], prm[2:2 + dims], prm[5:5 + dims], float(prm[0]),
                                                    g["q"], g["draws"], float(prm[1]))["near1"])


def test_grid_queries_match_oracle_large():
    x = wl.ball(200_000, 51)
    mn, mx = wl.bounds_for(x)
    rng = np.random.default_rng(52)
    q = rng.uniform(mn[0], mx[0], (20_000, 3)).astype(np.float32)
    draws = rng.integers(0, 2 ** 32, len(q), dtype=np.uint64).astype(np.uint32)
    grid = tg.Grid(3, mn, mx, 1.0, len(x))
    grid.rebuild(x)
    out = run_all(grid, q, draws, 1.7, len(x))
    ref = oracle.grid_query(x, mn, mx, 1.0, q, draws, 1.7)
    for k in out:
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)


def test_grid_edge_cases():
    # an empty grid answers -1; a point outside the bounds is clamped into an edge bin
    grid = tg.Grid(3, (-2, -2, -2), (2, 2, 2), 1.0, 8)
    grid.rebuild(np.zeros((0, 3), np.float32))
    assert (grid.nearest(np.zeros((3, 3), np.float32)) == -1).all()
    pts = np.array([[5.0, 5.0, 5.0], [0.1, 0.1, 0.1]], np.float32)
    grid.rebuild(pts)
    assert grid.nearest(np.array([[1.9, 1.9, 1.9]], np.float32), 0)[0] == 0
    with pytest.raises(tg.TecsError):
        grid.rebuild(np.zeros((9, 3), np.float32))
