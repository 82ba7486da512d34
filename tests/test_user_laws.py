"""User pairwise laws: PAIRWISE_FORCE lambdas and PAIRWISE_FORCE_OP functors.

tests/cpp/user_law_driver.cu writes the reference fixtures' two-radius spring
as a lambda (and once as a functor) with the operations of the reference's own
lambda, and is compiled by nvcc against include/tecs/pairwise.cuh.  The
library runs its force passes through the law compiled into the program
(tecs_sim_set_pair_law), so on a GB300 the program must reproduce the
reference's outputs exactly as the built-in law does: pair lists and runs bit
for bit, and the COM fix within the parity tolerance
(|gpu - ref| <= 1e-5 |ref| + 1e-6 rms(ref)).
"""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import tecs_gb300 as tg

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
SOURCE = Path(__file__).resolve().parent / "cpp" / "user_law_driver.cu"
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def build(out: Path) -> Path:
    if not Path(NVCC).exists():
        pytest.skip("nvcc not available")
    lib = Path(tg.library_path())
    cmd = [NVCC, "-std=c++20", "--extended-lambda", "-fmad=false", "-gencode", "arch=compute_103a,code=sm_103a",
           "-Xcompiler", "-Wall,-Wextra", f"-I{ROOT / 'include'}", str(SOURCE), f"-L{lib.parent}",
           "-l" + lib.stem[3:], "-Xlinker", f"-rpath,{lib.parent}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return out


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    return build(tmp_path_factory.mktemp("user_law") / "user_law_driver")


def write_input(path, g):
    x0 = g["x0"]
    p0 = g.get("p0")
    with open(path, "wb") as f:
        np.array([len(x0), x0.shape[1], 0 if p0 is None else 1], np.uint32).tofile(f)
        g["prm"].astype(np.float32).tofile(f)
        x0.astype(np.float32).tofile(f)
        if p0 is not None:
            p0.astype(np.float32).tofile(f)
        if "links" in g:
            np.array([len(g["links"])], np.uint32).tofile(f)
            g["links"].astype(np.uint32).tofile(f)


def run(driver, scenario, name, tmp_path, steps=None):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    inp = tmp_path / "in.bin"
    write_input(inp, g)
    out = tmp_path / "out"
    k = int(g["steps"]) if steps is None else steps
    r = subprocess.run([str(driver), scenario, str(inp), str(out), str(k), repr(float(g["dt"]))],
                       capture_output=True, text=True, timeout=600, cwd=tmp_path)
    return g, out, r


def close(a, b, rtol=1e-5, atol=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.sqrt(np.mean(b ** 2)) if b.size else 0.0
    return bool((np.abs(a - b) <= rtol * np.abs(b) + atol * scale).all())


def test_user_law_program_builds_and_fails_cleanly_without_a_device(tmp_path):
    """The header compiles with the program's laws under nvcc; with no GPU the library's error surfaces."""
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    exe = build(tmp_path / "user_law_driver")
    _, _, r = run(exe, "bg_heun", "bg_heun", tmp_path)
    assert r.returncode == 1 and "tecs error" in r.stderr


def test_counter_random_is_reproducible_and_well_distributed(tmp_path):
    """tests/cpp/random_checks.cpp: the generator user laws draw from (host build of the same code)."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "random_checks"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
                        str(SOURCE.parent / "random_checks.cpp"), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout


CASES = [
    # (scenario, fixture, exact)
    ("na_heun", "na_heun", True),
    ("ng_heun", "ng_heun", True),
    ("ba_euler", "c1_small_euler", True),
    ("bg_heun", "bg_heun", True),
    ("bg_heun", "bg_heun_clamped", True),
    ("bg_heun_functor", "bg_heun", True),
    ("bg_heun_2d", "bg_heun_2d", True),
    ("bg_heun_com", "bg_heun_com", False),
    ("bg_heun_pol", "bg_heun_polarity", False),
]


@pytest.mark.gpu
@pytest.mark.parametrize("scenario,name,exact", CASES)
def test_user_law_reproduces_reference(driver, tmp_path, scenario, name, exact):
    g, out, r = run(driver, scenario, name, tmp_path)
    assert r.returncode == 0, r.stderr
    dims = g["x0"].shape[1]
    pairs = np.fromfile(f"{out}.pairs", np.uint32).reshape(-1, 2)
    np.testing.assert_array_equal(tg.canonical_pairs(pairs), tg.canonical_pairs(g["pairs"]))
    dpos = np.fromfile(f"{out}.dpos", np.float32).reshape(-1, dims)
    pos = np.fromfile(f"{out}.pos", np.float32).reshape(-1, dims)
    if exact:
        np.testing.assert_array_equal(dpos, g["dpos"])
        np.testing.assert_array_equal(pos, g["pos"])
    else:
        assert close(dpos, g["dpos"]) and close(pos, g["pos"])
    if "pol" in g:
        assert close(np.fromfile(f"{out}.pol", np.float32).reshape(-1, 2), g["pol"])


@pytest.mark.gpu
def test_user_law_with_links_reproduces_reference(driver, tmp_path):
    """take_step(dt, forces::LinkPull, PAIRWISE_FORCE(...)()): links after the user law, bit for bit."""
    g, out, r = run(driver, "lk_bg_heun", "lk_bg_heun", tmp_path)
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(np.fromfile(f"{out}.pos", np.float32).reshape(-1, 3), g["pos"])


@pytest.mark.gpu
@pytest.mark.parametrize("scenario,name,exact", [("lk_lambda_bg_heun", "lk_bg_heun", True),
                                                 ("lk_lambda_ba_euler_com", "lk_ba_euler_com", False)])
def test_link_force_lambda_reproduces_reference(driver, tmp_path, scenario, name, exact):
    """take_step(dt, LINK_FORCE(...)(), PAIRWISE_FORCE(...)()): the protrusion law written as the reference's
    programs write it, evaluated per link end after the pair sums in link order; bit for bit against the
    reference's link runs (within the COM tolerance with the COM fix)."""
    g, out, r = run(driver, scenario, name, tmp_path)
    assert r.returncode == 0, r.stderr
    pos = np.fromfile(f"{out}.pos", np.float32).reshape(-1, 3)
    if exact:
        np.testing.assert_array_equal(pos, g["pos"])
    else:
        assert close(pos, g["pos"])


@pytest.mark.gpu
@pytest.mark.parametrize("name,exact", [("fields_bg_heun", True), ("fields_ba_euler_com", False)])
def test_config_with_extra_fields_reproduces_reference(driver, tmp_path, name, exact):
    """CONFIG_FIELDS((Vector, position), (Scalar, u), (Vector, w)): laws that read and write u and w through
    ctx, and the integrators updating every field (the Scalar field in double, as the reference's float +=
    float * double dt).  Ten steps bit for bit against the reference's run (within the COM tolerance with
    the COM fix, which moves the positions and so the w term of the law)."""
    g, out, r = run(driver, name, name, tmp_path)
    assert r.returncode == 0, r.stderr
    pos = np.fromfile(f"{out}.pos", np.float32).reshape(-1, 3)
    u = np.fromfile(f"{out}.u", np.float32)
    w = np.fromfile(f"{out}.w", np.float32).reshape(-1, 3)
    assert not np.array_equal(u, g["x0"][:, 0] * np.float32(0.3) + np.float32(1))  # u evolved
    if exact:
        np.testing.assert_array_equal(pos, g["pos"])
        np.testing.assert_array_equal(u, g["u"])
        np.testing.assert_array_equal(w, g["w"])
    else:
        assert close(pos, g["pos"]) and close(u, g["u"]) and close(w, g["w"])


@pytest.mark.gpu
def test_generic_law_with_pairwise_law_reproduces_reference(driver, tmp_path):
    """take_step(dt, PAIRWISE_FORCE(...)(), GENERIC_FORCE(...)()): the generic law (is_full_step-dependent,
    reading ctx.position.self) is added before the pair sums, as the reference fuses them; bit for bit."""
    g, out, r = run(driver, "gen_bg_heun", "gen_bg_heun", tmp_path)
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(np.fromfile(f"{out}.pos", np.float32).reshape(-1, 3), g["pos"])


@pytest.mark.gpu
def test_user_law_random_draws_are_reproducible(driver, tmp_path):
    """A law drawing from rng gives the same run twice, and a run that differs from the plain spring's."""
    g, out, r = run(driver, "rng_twice", "bg_heun", tmp_path, steps=5)
    assert r.returncode == 0, r.stderr
    a = np.fromfile(f"{out}.a.pos", np.float32).reshape(-1, 3)
    b = np.fromfile(f"{out}.b.pos", np.float32).reshape(-1, 3)
    np.testing.assert_array_equal(a, b)
    assert np.isfinite(a).all() and not np.array_equal(a, g["x0"])


@pytest.mark.gpu
@pytest.mark.parametrize("name,exact", [("drag_bg_heun", True), ("drag_ba_euler_com", False)])
def test_user_law_setting_drag_reproduces_reference(driver, tmp_path, name, exact):
    """A law that sets drag: each cell's position delta gains sum(drag * old velocity of j) /
    max(sum(drag), eps) (binned_gabriel.hpp:225-226, 356-357), with the old velocities the
    integrators write every step (euler.hpp:59, heun.hpp:87).  Positions and old velocities after
    8 steps: bit for bit without the COM fix, within the COM tolerance with it."""
    g, out, r = run(driver, name, name, tmp_path)
    assert r.returncode == 0, r.stderr
    pos = np.fromfile(f"{out}.pos", np.float32).reshape(-1, 3)
    ov = np.fromfile(f"{out}.ov", np.float32).reshape(-1, 3)
    assert np.abs(g["ov"]).max() > 0.1
    if exact:
        np.testing.assert_array_equal(pos, g["pos"])
        np.testing.assert_array_equal(ov, g["ov"])
    else:
        # the COM sum's last bits move the positions by ~1e-6; the old
        # velocities are forces at those positions (spring stiffness 2, drag
        # weights up to 0.6), so they agree to ~1e-5 absolute
        assert close(pos, g["pos"])
        assert close(ov, g["ov"], rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
def test_naive_delaunay_program_past_4096_cells_of_capacity(driver, tmp_path):
    """A 2-D NaiveDelaunay program with a user law: up to 4096 cells of capacity the library runs the naive
    finder, past that its Delaunay finder of any capacity (the user law's pass for FINDER 5).  The same cells
    give the same pairs with the same multiplicities, deltas and 5-step Euler run either way, bit for bit."""
    rng = np.random.default_rng(12)
    n = 1200
    r = np.sqrt(rng.random(n) * n / np.pi)
    t = rng.random(n) * 2 * np.pi
    x0 = np.stack([r * np.cos(t), r * np.sin(t)], 1).astype(np.float32)
    outs = []
    for cap in (n, 5000):
        prm = np.zeros(16, np.float32)
        prm[0] = 1.0                      # cutoff
        prm[8:12] = (2.0, 0.7, 0.5, 0.8)  # the spring
        prm[13] = cap
        prm[14] = 1.0
        g = {"x0": x0, "prm": prm}
        d = tmp_path / f"cap{cap}"
        d.mkdir()
        inp = d / "in.bin"
        write_input(inp, g)
        out = d / "out"
        res = subprocess.run([str(driver), "nd_euler_2d", str(inp), str(out), "5", "0.05"], capture_output=True,
                             text=True, timeout=600, cwd=d)
        assert res.returncode == 0, res.stderr
        outs.append({k: np.fromfile(f"{out}.{k}", np.uint32 if k == "pairs" else np.float32)
                     for k in ("pairs", "dpos", "pos")})
    a, b = outs
    pa = np.sort(a["pairs"].reshape(-1, 2).view(np.uint64).ravel())
    pb = np.sort(b["pairs"].reshape(-1, 2).view(np.uint64).ravel())
    assert len(pa) > 2 * n and len(np.unique(pa)) < len(pa)  # pairs repeat once per accepted triangle
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(a["dpos"], b["dpos"])
    np.testing.assert_array_equal(a["pos"], b["pos"])
