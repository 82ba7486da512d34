"""The Delaunay finder of any capacity, on the CPU (tecs/device/delaunay_star.cuh).

The header is compiled for the host (tests/cpp/delaunay_star_host.cpp) and
checked against:
  * 2-D: the naive restatement of naive_delaunay.hpp:45-99 (oracle/), bit for
    bit -- every pair and its number of applications -- on random, clustered,
    far-from-origin, jittered and exact lattice inputs, with duplicates and a
    collinear row;
  * 3-D: the reference's counting rule applied to an independent Delaunay
    triangulation (Qhull, through scipy): for each tetrahedron (i, j, k, l),
    the pair (i, j) in cutoff once per distinct k = min(k, l).
The reference's 3-D sphere is centred at x_i + c (c the circumcentre) rather
than at c; a test below pins that reading of naive_delaunay.hpp:187-214 on the
oracle, and shows that its multiplicities are not those of any triangulation.
"""
import collections
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle

ROOT = Path(__file__).resolve().parents[1]
SOURCE = ROOT / "tests" / "cpp" / "delaunay_star_host.cpp"


@pytest.fixture(scope="module")
def star_bin(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("dl") / "star"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
                    f"-I{ROOT / 'include'}", str(SOURCE), "-o", str(out)], check=True)
    return out


def star(binary, x, cutoff):
    """{(i, j): reps} and the OR of the cells' error bits."""
    n, dims = x.shape
    xx = np.zeros((n, 3), np.float32)
    xx[:, :dims] = x
    text = f"{n} {dims} {float(np.float32(cutoff))!r}\n" + "".join(
        " ".join("%.9g" % float(v) for v in r) + "\n" for r in xx)
    out = subprocess.run([str(binary)], input=text, capture_output=True, text=True, check=True).stdout
    res, err = {}, None
    for ln in out.splitlines():
        f = ln.split()
        if f[0] == "err":
            err = int(f[1])
        elif f[0] != "cellerr":
            res[(int(f[0]), int(f[1]))] = int(f[2])
    return res, err


def naive(x, cutoff):
    o = oracle.Oracle(dims=x.shape[1], finder=oracle.NAIVE_DELAUNAY, cutoff=cutoff, min_bounds=(-1e3,) * 3,
                      max_bounds=(1e3,) * 3, integrator=oracle.EULER, capacity=len(x))
    o.set_state(x)
    return dict(collections.Counter(map(tuple, o.evaluate()[2].tolist())))


def qhull_counts(x, cutoff):
    spatial = pytest.importorskip("scipy.spatial")
    tri = spatial.Delaunay(x.astype(np.float64))
    rc2 = np.float32(cutoff) * np.float32(cutoff)
    ks = collections.defaultdict(set)
    for s in tri.simplices.tolist():
        for i in s:
            for j in s:
                if j == i:
                    continue
                d = x[i] - x[j]
                d2 = (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]
                if d2 < rc2:
                    ks[(i, j)].add(min(v for v in s if v != i and v != j))
    return {key: len(v) for key, v in ks.items()}


def inputs_2d(kind, rng):
    if kind == "disk":
        r = np.sqrt(rng.random(150)) * 4
        t = rng.random(150) * 2 * np.pi
        return np.stack([r * np.cos(t), r * np.sin(t)], 1)
    if kind == "far":
        return rng.random((200, 2)) * 5 + 40
    if kind == "jittered_lattice":
        g = np.stack(np.meshgrid(np.arange(12), np.arange(12), indexing="ij"), -1).reshape(-1, 2) * 0.8
        return g + rng.normal(0, 1e-3, g.shape)
    if kind == "hex_lattice":
        pts = [(i + 0.5 * (j % 2), j * np.sqrt(3) / 2) for i in range(10) for j in range(10)]
        return np.array(pts)[rng.permutation(100)]
    if kind == "clusters_duplicates":
        c = rng.random((8, 2)) * 6
        x = c[rng.integers(0, 8, 120)] + rng.normal(0, 0.3, (120, 2))
        x[5] = x[17]
        x[40] = x[41]
        return x
    # exact square lattice (four cocircular points per square) and a collinear row
    g = np.stack(np.meshgrid(np.arange(9), np.arange(9), indexing="ij"), -1).reshape(-1, 2) * 0.5
    return np.concatenate([g, np.stack([np.linspace(-3, 7, 10), np.full(10, -1.0)], 1)])


KINDS_2D = ["disk", "far", "jittered_lattice", "hex_lattice", "clusters_duplicates", "lattice_and_row"]


@pytest.mark.parametrize("kind", KINDS_2D)
@pytest.mark.parametrize("cutoff", [0.6, 2.5, 100.0])
def test_2d_multiplicities_are_the_naive_finders(star_bin, kind, cutoff):
    x = inputs_2d(kind, np.random.default_rng(KINDS_2D.index(kind))).astype(np.float32)
    got, err = star(star_bin, x, cutoff)
    want = naive(x, cutoff)
    assert err & ~2 == 0  # bit 2 (a full near-circle list) only reorders which far points are kept
    assert got == want
    if cutoff == 100.0 and kind == "disk":
        assert max(want.values()) == 2  # an interior edge borders two triangles
    if cutoff == 100.0 and kind == "far":
        # 40 units from the origin the float circumcentre (from |x|^2 terms) is
        # off by ~1e-4, and rounding accepts a third triangle on some edges
        assert max(want.values()) == 3


def test_2d_degenerate_inputs(star_bin):
    # fewer than three cells, all collinear, all coincident: no triangle
    for x in ([[0, 0]], [[0, 0], [1, 0]], [[0, 0], [0.5, 0], [1.0, 0], [1.5, 0]], [[1, 1]] * 5):
        x = np.asarray(x, np.float32)
        got, err = star(star_bin, x, 10.0)
        assert got == naive(x, 10.0) == {} and err == 0


def ball(n, radius, seed, offset=0.0):
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    return (u * (rng.random(n) ** (1 / 3))[:, None] * radius + offset).astype(np.float32)


@pytest.mark.parametrize("case", ["ball", "far_slab", "clusters", "jittered_lattice", "all_in_cutoff"])
def test_3d_multiplicities_follow_the_delaunay_tetrahedra(star_bin, case):
    rng = np.random.default_rng(7)
    cutoff = 1.5
    if case == "ball":
        x = ball(1500, 7.0, 1)
    elif case == "far_slab":
        x = (rng.random((600, 3)) * np.array([10, 10, 1.0]) + 100).astype(np.float32)
    elif case == "clusters":
        c = rng.random((10, 3)) * 8
        x = (c[rng.integers(0, 10, 500)] + rng.normal(0, 0.5, (500, 3))).astype(np.float32)
    elif case == "jittered_lattice":
        g = np.stack(np.meshgrid(*[np.arange(7)] * 3, indexing="ij"), -1).reshape(-1, 3) * 0.9
        x = (g + rng.normal(0, 1e-2, g.shape)).astype(np.float32)
    else:
        x, cutoff = ball(300, 2.0, 3), 100.0
    got, err = star(star_bin, x, cutoff)
    assert err == 0
    assert got == qhull_counts(x, cutoff)


def test_3d_coplanar_cells_span_no_tetrahedron(star_bin):
    g = np.stack(np.meshgrid(np.arange(6), np.arange(6), indexing="ij"), -1).reshape(-1, 2) * 0.7
    x = np.concatenate([g, np.zeros((36, 1))], 1).astype(np.float32)
    got, err = star(star_bin, x, 2.0)
    assert got == {} and err == 0
    assert naive(x, 2.0) == {}  # every determinant is exactly zero for the reference too


def test_reference_3d_sphere_is_centred_at_xi_plus_the_circumcentre():
    # naive_delaunay.hpp:187-214 solves 2 (x_m - x_i).c = |x_m|^2 - |x_i|^2 for
    # c (the circumcentre itself) and then adds x_i: on the oracle, a cell i
    # far from the origin with three close neighbours gets the pair applied
    # exactly when the ball of radius |c| about x_i + c holds no other point
    pts = np.array([[10.0, 0, 0], [10.5, 0, 0], [10.0, 0.5, 0], [10.0, 0, 0.5]], np.float32)
    e = (pts[1:] - pts[0]).astype(np.float64)
    b = (pts[1:].astype(np.float64) ** 2).sum(1) - (pts[0].astype(np.float64) ** 2).sum()
    c = np.linalg.solve(2 * e, b)
    assert np.allclose(np.linalg.norm(pts - c, axis=1), np.linalg.norm(pts[0] - c))  # the circumcentre
    centre, radius = pts[0] + c, np.linalg.norm(c)  # the reference's sphere: through i, not through j
    assert abs(np.linalg.norm(pts[1] - centre) - radius) > 0.4
    # a fifth point inside the reference's sphere (far from the tetrahedron) removes the pair;
    # outside it, the pair is applied -- the circumsphere itself is the same in both
    inside = (centre + 0.1 * (pts[0] - centre)).astype(np.float32)
    outside = np.array([-10.0, 0, 0], np.float32)
    base = naive(pts, 1.0)
    with_inside = naive(np.concatenate([pts, inside[None]]), 1.0)
    with_outside = naive(np.concatenate([pts, outside[None]]), 1.0)
    assert base.get((0, 1), 0) >= 1 and with_outside.get((0, 1), 0) >= 1
    assert with_inside.get((0, 1), 0) == 0


def test_reference_3d_multiplicities_exceed_any_triangulation():
    # around an edge, a triangulation has a ring of a handful of tetrahedra;
    # the reference's 3-D test accepts far more third points on random input
    x = ball(60, 1.0, 4)
    want = naive(x, 1.0)
    ring = qhull_counts(x, 1.0)
    assert max(want.values()) > 3 * max(ring.values())
