"""The Delaunay finder of any capacity on a GB300 (finder "delaunay": k_dl_* kernels).

* 2-D: the same pairs with the same multiplicities, the same deltas and the
  same Euler and Heun runs as the naive finder (k_delaunay_mult, pinned to the
  reference's fixtures), bit for bit;
* 3-D: the pairs follow the Delaunay tetrahedra of Qhull (scipy) under the
  reference's counting rule;
* 100k cells: in 2-D every cell's row equals that of the same search
  compiled for the host (tests/cpp/delaunay_star_host.cpp), in 3-D Qhull's;
  Heun steps run without an overflow.
"""
import collections
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import tecs_gb300 as tg

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def make(x, finder, integrator="euler", cutoff=1.0):
    n, dims = x.shape
    pf = tg.PairFinderSettings(min_bounds=(-1e3,) * 3, max_bounds=(1e3,) * 3)
    s = tg.Simulation(tg.Settings(agent_count=n, capacity=n, cutoff_distance=cutoff, pair_finder_settings=pf),
                      dims=dims, pair_finder=finder, integrator=integrator, force=tg.Spring2R())
    s.set_state(x)
    return s


def counts(pairs):
    return dict(collections.Counter(map(tuple, np.asarray(pairs).tolist())))


def disk(n, seed, density=1.0):
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.random(n) * n / (np.pi * density))
    t = rng.random(n) * 2 * np.pi
    return np.stack([r * np.cos(t), r * np.sin(t)], 1).astype(np.float32)


def ball(n, seed, density=1.0):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    radius = (3 * n / (4 * np.pi * density)) ** (1 / 3)
    return (u * (rng.random(n) ** (1 / 3))[:, None] * radius).astype(np.float32)


def inputs_2d(kind):
    rng = np.random.default_rng(11)
    if kind == "disk":
        return disk(700, 1)
    if kind == "far":
        return (rng.random((500, 2)) * 18 + 60).astype(np.float32)
    if kind == "clusters_duplicates":
        c = rng.random((12, 2)) * 14
        x = (c[rng.integers(0, 12, 600)] + rng.normal(0, 0.6, (600, 2))).astype(np.float32)
        x[3] = x[30]
        x[100] = x[101]
        return x
    g = np.stack(np.meshgrid(np.arange(22), np.arange(22), indexing="ij"), -1).reshape(-1, 2) * 0.7
    return g.astype(np.float32)  # exact square lattice: four cocircular points per square


@pytest.mark.parametrize("kind", ["disk", "far", "clusters_duplicates", "lattice"])
@pytest.mark.parametrize("cutoff", [1.0, 2.5])
def test_2d_same_pairs_deltas_and_runs_as_the_naive_finder(kind, cutoff):
    x = inputs_2d(kind)
    a, b = make(x, "delaunay", cutoff=cutoff), make(x, "naive_delaunay", cutoff=cutoff)
    da, _, pa = a.evaluate()
    db, _, pb = b.evaluate()
    assert counts(pa) == counts(pb) and len(pb) > 0
    np.testing.assert_array_equal(da, db)
    a.take_step(0.05, 3)
    b.take_step(0.05, 3)
    np.testing.assert_array_equal(a.get_state()[0], b.get_state()[0])


def test_2d_heun_runs_as_the_naive_finder():
    x = disk(900, 4)
    a, b = make(x, "delaunay", "heun"), make(x, "naive_delaunay", "heun")
    a.take_step(0.05, 4)
    b.take_step(0.05, 4)
    np.testing.assert_array_equal(a.get_state()[0], b.get_state()[0])


def qhull_counts(x, cutoff):
    spatial = pytest.importorskip("scipy.spatial")
    S = spatial.Delaunay(x.astype(np.float64)).simplices
    rc2 = np.float32(cutoff) * np.float32(cutoff)
    out = []
    for a in range(4):
        for b in range(4):
            if a == b:
                continue
            rest = [c for c in range(4) if c not in (a, b)]
            i, j = S[:, a], S[:, b]
            k = np.minimum(S[:, rest[0]], S[:, rest[1]])
            d = x[i] - x[j]
            d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
            m = d2 < rc2
            out.append(np.stack([i[m], j[m], k[m]], 1))
    ijk = np.unique(np.concatenate(out), axis=0)
    ij, c = np.unique(ijk[:, :2], axis=0, return_counts=True)
    return {(int(p), int(q)): int(v) for (p, q), v in zip(ij, c)}


def test_3d_pairs_follow_the_delaunay_tetrahedra():
    x = ball(4000, 2)
    s = make(x, "delaunay", cutoff=1.5)
    assert counts(s.evaluate()[2]) == qhull_counts(x, 1.5)


@pytest.fixture(scope="module")
def host_star(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("dl") / "star"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "delaunay_star_host.cpp"), "-o", str(out)], check=True)
    return out


def host_rows(binary, x, cutoff):
    n, dims = x.shape
    xx = np.zeros((n, 3), np.float32)
    xx[:, :dims] = x
    text = f"{n} {dims} {float(np.float32(cutoff))!r}\n" + "\n".join(
        " ".join("%.9g" % float(v) for v in r) for r in xx) + "\n"
    out = subprocess.run([str(binary)], input=text, capture_output=True, text=True, check=True).stdout
    rows = {}
    for ln in out.splitlines():
        f = ln.split()
        if f[0] == "err":
            assert int(f[1]) & ~2 == 0
        elif f[0] != "cellerr":
            rows[(int(f[0]), int(f[1]))] = int(f[2])
    return rows


@pytest.mark.parametrize("dims", [2, 3])
def test_100k_cells_rows_and_heun_steps(host_star, dims):
    n = 100_000
    x = disk(n, 5) if dims == 2 else ball(n, 6)
    s = make(x, "delaunay", "heun", cutoff=1.5)
    got = counts(s.evaluate()[2])
    if dims == 2:
        assert got == host_rows(host_star, x, 1.5)
    else:
        assert got == qhull_counts(x, 1.5)
        # the tetrahedra around an edge are the same from either end
        assert all(got.get((j, i)) == r for (i, j), r in got.items())
    per_cell = np.bincount(np.array(list(got))[:, 0], minlength=n)
    # a few cells on the rim have no Delaunay neighbour within the cutoff
    assert (per_cell == 0).mean() < 1e-3 and per_cell.mean() > (4 if dims == 2 else 8)
    s.take_step(0.02, 3)
    y, _ = s.get_state()
    assert np.isfinite(y).all() and np.abs(y - x).max() < 1.0


def test_finder_rejects_symmetric():
    x = disk(50, 2)
    pf = tg.PairFinderSettings(min_bounds=(-1e3,) * 3, max_bounds=(1e3,) * 3)
    with pytest.raises(tg.TecsError):
        tg.Simulation(tg.Settings(agent_count=50, capacity=50, cutoff_distance=1.0, pair_finder_settings=pf),
                      dims=2, pair_finder="delaunay", symmetric=True, force=tg.Spring2R())
