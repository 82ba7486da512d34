"""Pin the oracle (C restatement) to the TECS reference.

The fixtures in tests/golden/ were produced by the reference's own headers,
compiled unmodified against oracle/kokkos_shim (tests/golden/make_golden.py).
The restatement must reproduce them bit for bit: the directed pair lists in the
reference's evaluation order, the per-cell deltas of one full-step pass, and
the state after the recorded number of Simulation::take_step calls.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
MANIFEST = json.loads((GOLDEN / "manifest.json").read_text())

# name -> (finder, symmetric, integrator, com, dims, polarity), mirrors make_golden.SCENARIOS
KIND = {
    "c1_small_euler": (1, 0, 0, 0, 3, 0),
    "bg_heun": (3, 0, 1, 0, 3, 0),
    "bg_heun_com": (3, 0, 1, 1, 3, 0),
    "bg_heun_clamped": (3, 0, 1, 0, 3, 0),
    "ba_heun_com": (1, 0, 1, 1, 3, 0),
    "bg_euler_com": (3, 0, 0, 1, 3, 0),
    "na_heun": (0, 0, 1, 0, 3, 0),
    "ng_heun": (2, 0, 1, 0, 3, 0),
    "bgs_euler_com": (3, 1, 0, 1, 3, 0),
    "bas_heun": (1, 1, 1, 0, 3, 0),
    "ngs_euler": (2, 1, 0, 0, 3, 0),
    "nas_heun": (0, 1, 1, 0, 3, 0),
    "bg_heun_polarity": (3, 0, 1, 0, 3, 1),
    "ng_euler_2d_points11": (2, 0, 0, 0, 2, 0),
    "bg_heun_2d": (3, 0, 1, 0, 2, 0),
    "nd_euler_2d": (4, 0, 0, 0, 2, 0),
    "nd_euler_2d_points11": (4, 0, 0, 0, 2, 0),
    "nd_heun_3d": (4, 0, 1, 0, 3, 0),
    "lk_bg_heun": (3, 0, 1, 0, 3, 0),
    "lk_ba_euler_com": (1, 0, 0, 1, 3, 0),
}
# fixtures of the link-force scenarios hold the final state only
LINKED = sorted(k for k in KIND if k.startswith("lk_"))
# fixtures of the reference's HDF5_Writer: the inputs and the XDMF sidecar
# (tests/test_cpp_drop_in.py compares the drop-in writer's with it)
WRITER = ["lk_writer", "lk_writer_nolinks"]
# fixtures of a GENERIC_FORCE law with the spring: the reference's final state,
# which the user-law program reproduces on a GPU (tests/test_user_laws.py);
# the C restatement has built-in laws only
USER_LAW = ["gen_bg_heun", "drag_bg_heun", "drag_ba_euler_com", "upd_bg_heun", "fields_bg_heun",
            "fields_ba_euler_com"]
# fixtures of the reference's standalone acceleration::Grid queries
GRID = ["grid_q_3d", "grid_q_2d"]
# output of five of the reference's example programs run on its headers
# (tests/test_reference_examples.py compares the drop-in layer's runs with it)
EXAMPLES = ["ex_springs", "ex_epithelium", "ex_polarization", "ex_growth_w_wall", "ex_delaunay_spheroid"]
# the reference's predefined force functions at a table of distances
# (tests/test_force_laws.py)
LAWS = ["laws_predefined"]


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def make_oracle(name, g, kind=None):
    finder, sym, integ, com, dims, pol = kind or KIND[name]
    prm = g["prm"]
    n = len(g["x0"])
    cap = max(int(prm[13]), n)
    o = oracle.Oracle(dims=dims, finder=finder, symmetric=bool(sym), cutoff=float(prm[0]),
                      gabriel_coefficient=float(prm[1]), min_bounds=tuple(prm[2:5]), max_bounds=tuple(prm[5:8]),
                      bin_size_scale=float(prm[14]), integrator=integ, com_fix=bool(com),
                      force=oracle.FORCE_POLARITY if pol else oracle.FORCE_SPRING2R, k_rep=float(prm[8]),
                      r_rep=float(prm[9]), k_adh=float(prm[10]), r_adh=float(prm[11]), k_pol=float(prm[12]),
                      has_polarity=bool(pol), capacity=cap)
    o.set_state(g["x0"], g.get("p0"))
    if "links" in g:
        o.set_links(g["links"], float(prm[15]))
    return o


def test_manifest_covers_every_fixture():
    assert set(MANIFEST) == set(KIND) | set(WRITER) | set(USER_LAW) | set(GRID) | set(EXAMPLES) | set(LAWS)
    for name in USER_LAW + GRID + EXAMPLES + LAWS:
        assert (GOLDEN / f"{name}.npz").exists()
    for name in list(KIND) + WRITER:
        assert (GOLDEN / f"{name}.npz").exists()
    for name in WRITER:
        assert (GOLDEN / f"{name}.xmf").read_bytes().startswith(b'<?xml version="1.0"?>\n<Xdmf Version="3.0">')


@pytest.mark.parametrize("name", sorted(set(KIND) - set(LINKED)))
def test_pairs_and_deltas_match_reference(name):
    g = load(name)
    o = make_oracle(name, g)
    dx, dp, pairs = o.evaluate()
    assert len(g["pairs"]) == MANIFEST[name]["pairs"]
    # the directed pair list in the reference's Serial evaluation order
    np.testing.assert_array_equal(pairs, g["pairs"])
    np.testing.assert_array_equal(dx, g["dpos"])
    if "dpol" in g:
        np.testing.assert_array_equal(dp, g["dpol"])


@pytest.mark.parametrize("name", sorted(KIND))
def test_steps_match_reference(name):
    g = load(name)
    o = make_oracle(name, g)
    o.step(float(g["dt"]), int(g["steps"]))
    x, p = o.get_state()
    np.testing.assert_array_equal(x, g["pos"])
    if "pol" in g:
        np.testing.assert_array_equal(p, g["pol"])


def test_points11_gabriel_neighbour_counts():
    # main.cpp's 2-D demo counts Gabriel neighbours per cell over both pair directions
    g = load("ng_euler_2d_points11")
    pairs = g["pairs"]
    counts = np.bincount(pairs[:, 0], minlength=11)
    # the graph is undirected: every (i, j) appears with (j, i)
    s = {tuple(p) for p in pairs.tolist()}
    assert all((j, i) in s for i, j in s)
    assert counts.sum() == len(pairs) and counts.min() >= 1


def test_delaunay_applies_a_pair_once_per_empty_simplex():
    # naive_delaunay.hpp applies (i, j) once per accepted triangle (2-D) or per
    # third point with an accepted tetrahedron (3-D): pairs repeat, and every
    # repeated application is still a directed pair within the cutoff
    for name in ("nd_euler_2d", "nd_heun_3d"):
        g = load(name)
        pairs = g["pairs"]
        uniq, counts = np.unique(pairs, axis=0, return_counts=True)
        assert counts.max() >= 2
        x = g["x0"]
        d2 = ((x[uniq[:, 0]] - x[uniq[:, 1]]) ** 2).sum(1)
        assert (d2 < float(g["prm"][0]) ** 2).all()
    # in 2-D an edge borders at most two triangles of points in general position
    u, c = np.unique(load("nd_euler_2d")["pairs"], axis=0, return_counts=True)
    assert c.max() <= 2


def test_link_fixtures_include_skipped_and_repeated_links():
    # the reference skips links with a == b and applies repeated links each time
    for name in LINKED:
        lk = load(name)["links"]
        assert (lk[:, 0] == lk[:, 1]).any()
        assert len(np.unique(lk, axis=0)) < len(lk)


def test_generic_force_fixture_is_the_spring_plus_the_generic_pull():
    # the same input under the spring alone ends elsewhere; the generic law pulls cells towards the
    # origin on full steps, so the reference's run ends more contracted
    g = load("gen_bg_heun")
    o = make_oracle("gen_bg_heun", g, kind=KIND["bg_heun"])
    o.step(float(g["dt"]), int(g["steps"]))
    spring_only, _ = o.get_state()
    assert np.isfinite(g["pos"]).all() and not np.array_equal(g["pos"], spring_only)
    assert np.sqrt((g["pos"] ** 2).sum(1)).mean() < np.sqrt((spring_only ** 2).sum(1)).mean()


@pytest.mark.parametrize("name", ["grid_q_3d", "grid_q_2d"])
def test_oracle_grid_queries_match_reference(name):
    # acceleration::Grid queried by the reference's own code (make_golden.py, GRID)
    g = load(name)
    prm = g["prm"]
    dims = g["x"].shape[1]
    out = oracle.grid_query(g["x"], prm[2:2 + dims], prm[5:5 + dims], float(prm[0]), g["q"], g["draws"],
                            float(prm[1]))
    for k in ("near1", "near2", "rbins", "rrad", "rfilt"):
        np.testing.assert_array_equal(out[k], g[k], err_msg=k)

