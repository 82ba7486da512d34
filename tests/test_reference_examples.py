"""The reference's example programs against the drop-in layer.

Two parts:

  * compile: nineteen of the reference's own programs (COMPILED, from its
    examples/) are copied byte for byte into a directory examples/ next to a
    link include/ -> this repository's include/, so that their
    "../include/tecs.hpp" is the drop-in layer's, and compiled by nvcc
    (-std=c++20 --extended-lambda) with the CUDA library.  This needs the
    reference checkout and runs where it is (no GPU needed to compile).
  * run: tests/cpp/example_programs.cu runs five of these experiments -- the
    same settings, initialisers, force laws, init and update functions,
    device values, steps and writes -- through the same API on a GB300, and
    its HDF5 output is compared with the reference programs' own output, made
    by running them on the reference's headers (tests/golden/make_golden.py,
    EXAMPLES):
      - the snapshot count and every snapshot's agent count: exact
        (growth_w_wall divides at random; its draws come from the same
        generator stream in the same order, so its cell counts must agree
        step for step);
      - the first snapshot (the initialisers' output): within 1e-6 relative --
        the initialisers run on the host from the reference's generator
        stream; libm may differ in the last bit between the machine that made
        the fixtures and the one running the test (epithelium writes first
        after one step of its polarity law: that law's 1e-5);
      - the last snapshot: positions within the parity tolerance where the run
        is short and smooth (springs), else by statistics (radius of gyration,
        mean neighbour count, polarity order), because the GPU's sums and the
        reference's differ in the last bit and long runs amplify that;
      - delaunay_spheroid: the links its pairwise law records from the
        Delaunay finder at t = 0, as a multiset, exactly.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np
import pytest

import oracle
import tecs_gb300 as tg
from tecs_gb300 import h5

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
# the programs run on a GB300 and compared with the reference's own runs
PROGRAMS = ["springs", "epithelium", "polarization", "growth_w_wall", "delaunay_spheroid"]
# every reference program that compiles unmodified against the drop-in layer:
# the five above, and programs using the other initialisers (line, cuboid,
# hexagon, rectangle, disk, relaxed cuboid), LINK_FORCE and UPDATE_FUNC with
# run / run_links, drag, set_capacity, extra int views, the polarity laws
# (apical constriction, migration), fields beyond the position and the
# polarity (Scalar fields, a second polarity), the host grid's random
# neighbour queries and the HDF5 reader
COMPILED = PROGRAMS + ["apical_constriction", "bending", "branching", "delaunay", "delaunay_sheet",
                       "epithelia_double_polarity", "gradient", "growth_w_squeeze", "intercalation",
                       "intercalation_w_gradient", "lineage_tracing", "migration", "passive_growth", "turing"]


def program_source(name):
    """The reference's program, read from the reference checkout."""
    ref = oracle.reference_root()
    if ref is None or not (ref / "examples" / f"{name}.cpp").exists():
        pytest.skip("the reference checkout is not present")
    return (ref / "examples" / f"{name}.cpp").read_bytes()


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    pytest.skip("nvcc not available")


def build(name, root):
    (root / "examples").mkdir(parents=True, exist_ok=True)
    if not (root / "include").exists():
        (root / "include").symlink_to(ROOT / "include")
    src = root / "examples" / f"{name}.cpp"
    src.write_bytes(program_source(name))
    lib = Path(tg.library_path())
    exe = root / "examples" / name
    cmd = [nvcc(), "-std=c++20", "--extended-lambda", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a",
           "-O2", "-fmad=false", str(src), f"-L{lib.parent}", "-l" + lib.stem[3:], "-Xlinker", "-rpath",
           "-Xlinker", str(lib.parent), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return exe, r


def test_programs_compile_unmodified(tmp_path):
    tg.load()
    with ThreadPoolExecutor(min(len(COMPILED), os.cpu_count() or 1)) as pool:
        results = list(pool.map(lambda n: build(n, tmp_path / n), COMPILED))
    for name, (exe, r) in zip(COMPILED, results):
        assert r.returncode == 0, (name, r.stderr[-3000:])
        assert exe.exists()


@pytest.fixture(scope="module")
def runs(tmp_path_factory):
    """The five experiments run once through tests/cpp/example_programs.cu;
    name -> (its HDF5 output, the reference program's fixture)."""
    lib = Path(tg.library_path())
    tg.load()
    root = tmp_path_factory.mktemp("programs")
    exe = root / "example_programs"
    src = Path(__file__).resolve().parent / "cpp" / "example_programs.cu"
    r = subprocess.run([nvcc(), "-std=c++20", "--extended-lambda", "-gencode", "arch=compute_103a,code=sm_103a", "-O2",
                        "-fmad=false", f"-I{ROOT / 'include'}", str(src), f"-L{lib.parent}", "-l" + lib.stem[3:],
                        "-Xlinker", "-rpath", "-Xlinker", str(lib.parent), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = {}
    for name in PROGRAMS:
        run_dir = root / name
        (run_dir / "output").mkdir(parents=True)
        p = subprocess.run([str(exe), name], cwd=run_dir, capture_output=True, text=True, timeout=900)
        assert p.returncode == 0, (name, p.stderr[-3000:])
        out[name] = (h5.H5File(run_dir / "output" / f"{name}.h5"), dict(np.load(GOLDEN / f"ex_{name}.npz")))
    return out


def snapshots(f):
    return sorted((int(k[1:]) for k in f.keys() if k.startswith("t")))


def close(a, b, rtol, atol_rms):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.sqrt(np.mean(b ** 2))
    err = np.abs(a - b)
    return bool(np.all(err <= rtol * np.abs(b) + atol_rms * scale)), float(err.max())


def radius_of_gyration(x):
    x = np.asarray(x, np.float64)
    return float(np.sqrt(((x - x.mean(0)) ** 2).sum(1).mean()))


def mean_neighbours(x, rc=1.0):
    from scipy.spatial import cKDTree

    x = np.asarray(x, np.float64)
    t = cKDTree(x)
    return float(np.mean([len(v) - 1 for v in t.query_ball_point(x, rc)]))


def polarity_order(p):
    th, ph = p[:, 0].astype(np.float64), p[:, 1].astype(np.float64)
    v = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
    return float(np.linalg.norm(v.sum(0)) / len(v))


# the first snapshot's tolerance: the initialisers' output (1e-6 relative),
# or for epithelium, whose first write follows one step of its polarity law,
# the parity tolerance of that law (CUDA's sin/cos/acos against libm's)
FIRST_TOL = {"epithelium": (1e-5, 1e-6)}


def check_counts_and_first(f, g, name):
    groups = snapshots(f)
    np.testing.assert_array_equal(groups, g["groups"])
    counts = [f.read(f"t{k}/position").shape[0] for k in groups]
    np.testing.assert_array_equal(counts, g["counts"])
    first = groups[0]
    rtol, atol = FIRST_TOL.get(name, (1e-6, 1e-7))
    ok, err = close(f.read(f"t{first}/position"), g[f"t{first}_position"], rtol, atol)
    assert ok, ("first snapshot", err)
    return groups


@pytest.mark.gpu
def test_springs_program(runs):
    f, g = runs["springs"]
    groups = check_counts_and_first(f, g, "springs")
    last = groups[-1]
    ok, err = close(f.read(f"t{last}/position"), g[f"t{last}_position"], 1e-5, 1e-6)
    assert ok, ("last snapshot", err)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["epithelium", "polarization"])
def test_polarity_programs(runs, name):
    f, g = runs[name]
    groups = check_counts_and_first(f, g, name)
    first, last = groups[0], groups[-1]
    rtol, atol = FIRST_TOL.get(name, (1e-6, 1e-7))
    ok, err = close(f.read(f"t{first}/polarity"), g[f"t{first}_polarity"], rtol, atol)
    assert ok, ("first polarity", err)
    x, xr = f.read(f"t{last}/position"), g[f"t{last}_position"]
    p, pr = f.read(f"t{last}/polarity"), g[f"t{last}_polarity"]
    assert abs(radius_of_gyration(x) - radius_of_gyration(xr)) <= 1e-3 * radius_of_gyration(xr)
    assert abs(mean_neighbours(x) - mean_neighbours(xr)) <= 0.02 * mean_neighbours(xr)
    assert abs(polarity_order(p) - polarity_order(pr)) <= 1e-2


@pytest.mark.gpu
def test_growth_w_wall_program(runs):
    f, g = runs["growth_w_wall"]
    groups = check_counts_and_first(f, g, "growth_w_wall")
    last = groups[-1]
    x, xr = f.read(f"t{last}/position"), g[f"t{last}_position"]
    assert len(x) == len(xr)
    assert abs(radius_of_gyration(x) - radius_of_gyration(xr)) <= 1e-2 * radius_of_gyration(xr)
    # the wall z = 0 holds the tissue on its positive side in both runs
    assert (x[:, 2] > -0.5).mean() == pytest.approx((xr[:, 2] > -0.5).mean(), abs=1e-3)


@pytest.mark.gpu
def test_delaunay_spheroid_program_links(runs):
    f, g = runs["delaunay_spheroid"]
    groups = snapshots(f)
    assert groups[0] == 0 and f.read("t0/position").shape[0] == 100
    ok, err = close(f.read("t0/position"), g["t0_position"], 1e-6, 1e-7)
    assert ok, ("first snapshot", err)
    links = f.read("t0/links")
    np.testing.assert_array_equal(tg.canonical_pairs(links), tg.canonical_pairs(g["t0_links"]))
