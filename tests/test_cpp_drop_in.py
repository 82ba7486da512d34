"""The C++20 drop-in layer (include/tecs/) against the reference's outputs.

tests/cpp/drop_in_driver.cpp is a program written the way the reference's
programs are (a config struct, Simulation<Config>, get_view, take_step); it is
compiled here with g++ against include/tecs/tecs.hpp and linked with the CUDA
library.  On a GB300 it runs on the inputs of the golden fixtures -- which hold
the reference's own outputs -- and must reproduce them: pair lists and spring
runs bit for bit, the COM fix and the polarity law within the parity
tolerance (|gpu - ref| <= 1e-5 |ref| + 1e-6 rms(ref)).
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import tecs_gb300 as tg

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
SOURCE = Path(__file__).resolve().parent / "cpp" / "drop_in_driver.cpp"


def link_flags():
    """The library the drop-in headers call (views hold device memory through it)."""
    lib = Path(tg.library_path())
    return [f"-L{lib.parent}", "-l" + lib.stem[3:], f"-Wl,-rpath,{lib.parent}"]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    lib = Path(tg.library_path())
    out = tmp_path_factory.mktemp("cpp") / "drop_in_driver"
    cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(SOURCE),
           f"-L{lib.parent}", "-l" + lib.stem[3:], f"-Wl,-rpath,{lib.parent}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_config_machinery_and_defaults(tmp_path):
    """tests/cpp/config_checks.cpp holds static_asserts on configs and Settings defaults."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = Path(__file__).resolve().parent / "cpp" / "config_checks.cpp"
    lib = Path(tg.library_path())
    out = tmp_path / "config_checks"
    r = subprocess.run(["g++", "-std=c++20", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(src),
                        f"-L{lib.parent}", "-l" + lib.stem[3:], f"-Wl,-rpath,{lib.parent}", "-o", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(out)], cwd=tmp_path).returncode == 0


def test_value_types_known_answers(tmp_path):
    """tests/cpp/value_types.cpp: the known answers of the reference's vector and polarity tests."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = Path(__file__).resolve().parent / "cpp" / "value_types.cpp"
    out = tmp_path / "value_types"
    r = subprocess.run(["g++", "-std=c++20", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(src),
                        *link_flags(), "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(out)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr


def test_hdf5_writer_matches_python_writer(tmp_path):
    """io::HDF5_Writer writes the same bytes as tecs_gb300.h5.H5Writer, and the reader reads them."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    import numpy as np
    from tecs_gb300 import h5

    src = Path(__file__).resolve().parent / "cpp" / "h5_writer.cpp"
    exe = tmp_path / "h5_writer"
    r = subprocess.run(["g++", "-std=c++20", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(src),
                        *link_flags(), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(exe), str(tmp_path / "cxx")], cwd=tmp_path).returncode == 0
    pos0 = np.array([[0.5 * i, -1.0 * i, 2.0 + i] for i in range(5)], np.float32)
    links = np.array([[l, 4 - l] for l in range(3)], np.uint32)
    pos1 = np.array([[1.0 + i, 0.25 * i, -0.5 * i] for i in range(7)], np.float32)
    pol1 = np.array([[np.float32(0.1) * np.float32(i), np.float32(-0.2) * np.float32(i)] for i in range(7)],
                    np.float32)
    w = h5.H5Writer(tmp_path / "py.h5")
    w.write_group("t0", {"position": pos0, "links": links})
    w.write_group("t1", {"position": pos1, "polarity": pol1})
    w.write_group("static", {"cell_type": np.array([[0], [1], [0], [1]], np.float32)})
    w.close()
    assert (tmp_path / "cxx.h5").read_bytes() == (tmp_path / "py.h5").read_bytes()
    f = h5.H5File(tmp_path / "cxx.h5")
    assert sorted(f.keys()) == ["static", "t0", "t1"]
    np.testing.assert_array_equal(f.read("t0/position"), pos0)
    np.testing.assert_array_equal(f.read("t0/links"), links)
    np.testing.assert_array_equal(f.read("t1/polarity"), pol1)


def test_hdf5_writer_long_run_matches_python_writer(tmp_path):
    """A write per step for 2,001 steps (t0 .. t2000, as the reference's bending example writes): the root
    group outgrows one B-tree node and its first name heap; both writers give the same bytes and every
    group reads back.  The writes hold the geometry alone, as sim.write(t) does."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    from tecs_gb300 import h5

    src = Path(__file__).resolve().parent / "cpp" / "h5_writer.cpp"
    exe = tmp_path / "h5_writer"
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
                        str(src), *link_flags(), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    steps = 2001
    assert subprocess.run([str(exe), str(tmp_path / "cxx"), str(steps)], cwd=tmp_path).returncode == 0

    def pos(s):
        return np.array([[s, -np.float32(s), np.float32(0.5) * np.float32(s)], [1.0, s % 7, -2.0]], np.float32)

    w = h5.H5Writer(tmp_path / "py.h5")
    for s in range(steps):
        w.write_group(f"t{s}", {"position": pos(s)})
    w.close()
    assert (tmp_path / "cxx.h5").read_bytes() == (tmp_path / "py.h5").read_bytes()
    f = h5.H5File(tmp_path / "cxx.h5")
    assert f.keys() == sorted(f"t{s}" for s in range(steps))
    for s in (0, 9, 10, 99, 100, 256, 257, 999, 1000, 1999, 2000):
        np.testing.assert_array_equal(f.read(f"t{s}/position"), pos(s))


@pytest.mark.parametrize("name", ["lk_writer", "lk_writer_nolinks"])
def test_xdmf_sidecar_matches_reference(tmp_path, name):
    """io::HDF5_Writer's "<path>.xmf" equals, byte for byte, the reference writer's sidecar for the
    same write sequence: write_static(cell_type), then (position, polarity, links) at t = 0, dt, 2 dt;
    with links the grids' topology is the links' polylines, without them the cells as vertices."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    src = Path(__file__).resolve().parent / "cpp" / "xdmf_writer.cpp"
    exe = tmp_path / "xdmf_writer"
    r = subprocess.run(["g++", "-std=c++20", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(src),
                        *link_flags(), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    args = [str(len(g["x0"])), str(len(g["links"])), str(int(g["steps"]) + 1), repr(float(g["dt"]))]
    assert subprocess.run([str(exe), str(tmp_path / "out"), *args], cwd=tmp_path).returncode == 0
    assert (tmp_path / "out.xmf").read_bytes() == (GOLDEN / f"{name}.xmf").read_bytes()


def write_input(path, g):
    x0 = g["x0"]
    p0 = g.get("p0")
    with open(path, "wb") as f:
        np.array([len(x0), x0.shape[1], 1 if p0 is not None else 0], np.uint32).tofile(f)
        g["prm"].astype(np.float32).tofile(f)
        x0.astype(np.float32).tofile(f)
        if p0 is not None:
            p0.astype(np.float32).tofile(f)
        if "links" in g:
            np.array([len(g["links"])], np.uint32).tofile(f)
            g["links"].astype(np.uint32).tofile(f)


def run_driver(driver, scenario, name, tmp_path):
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    inp = tmp_path / "in.bin"
    write_input(inp, g)
    out = tmp_path / "out"
    r = subprocess.run([str(driver), scenario, str(inp), str(out), str(int(g["steps"])), repr(float(g["dt"]))],
                       capture_output=True, text=True, timeout=600, cwd=tmp_path)
    return g, out, r


def test_driver_builds_and_fails_cleanly_without_a_device(driver, tmp_path):
    """Compiles with -Wall -Wextra -Werror; with no GPU the C ABI's error surfaces as tecs::Error."""
    import os

    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    _, _, r = run_driver(driver, "bg_heun", "bg_heun", tmp_path)
    assert r.returncode == 1
    assert "tecs error" in r.stderr


def close(a, b, rtol=1e-5, atol=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.sqrt(np.mean(b ** 2)) if b.size else 0.0
    return bool((np.abs(a - b) <= rtol * np.abs(b) + atol * scale).all())


CASES = [
    # (scenario in the driver, fixture, exact)
    ("ba_euler", "c1_small_euler", True),
    ("bg_heun", "bg_heun", True),
    ("bg_heun", "bg_heun_clamped", True),
    ("bg_heun_com", "bg_heun_com", False),
    ("bg_heun_pol", "bg_heun_polarity", False),
    ("nd_euler_2d", "nd_euler_2d", True),
    ("nd_euler_2d", "nd_euler_2d_points11", True),
]


@pytest.mark.gpu
@pytest.mark.parametrize("scenario,name,exact", CASES)
def test_drop_in_program_reproduces_reference(driver, tmp_path, scenario, name, exact):
    g, out, r = run_driver(driver, scenario, name, tmp_path)
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
        assert close(dpos, g["dpos"])
        assert close(pos, g["pos"])
    if "pol" in g:
        pol = np.fromfile(f"{out}.pol", np.float32).reshape(-1, 2)
        assert close(pol, g["pol"])


@pytest.mark.gpu
@pytest.mark.parametrize("name,exact", [("lk_bg_heun", True), ("lk_ba_euler_com", False)])
def test_drop_in_links_reproduce_reference(driver, tmp_path, name, exact):
    """get_links() + take_step(dt, forces::LinkPull, forces::Spring2R) against the reference's link runs."""
    g, out, r = run_driver(driver, name, name, tmp_path)
    assert r.returncode == 0, r.stderr
    pos = np.fromfile(f"{out}.pos", np.float32).reshape(-1, 3)
    if exact:
        np.testing.assert_array_equal(pos, g["pos"])
    else:
        assert close(pos, g["pos"])


@pytest.mark.gpu
def test_drop_in_program_writes_hdf5_snapshots(driver, tmp_path):
    """CONFIG_WRITER(io::HDF5_Writer): write(0), then take_step + write per step; the groups hold the trajectory."""
    from tecs_gb300 import h5

    g, out, r = run_driver(driver, "bg_heun_h5", "bg_heun", tmp_path)
    assert r.returncode == 0, r.stderr
    f = h5.H5File(f"{out}.h5")
    steps = int(g["steps"])
    assert sorted(f.keys(), key=lambda k: int(k[1:])) == [f"t{k}" for k in range(steps + 1)]
    np.testing.assert_array_equal(f.read("t0/position"), g["x0"])
    np.testing.assert_array_equal(f.read(f"t{steps}/position"), g["pos"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["lk_writer", "lk_writer_nolinks"])
def test_drop_in_program_writes_the_reference_xdmf(driver, tmp_path, name):
    """A stepped program with polarity, links and a static view: its "<out>.xmf" equals the
    reference's byte for byte, and every group it names is in "<out>.h5"."""
    from tecs_gb300 import h5

    g, out, r = run_driver(driver, "lk_writer", name, tmp_path)
    assert r.returncode == 0, r.stderr
    assert Path(f"{out}.xmf").read_bytes() == (GOLDEN / f"{name}.xmf").read_bytes()
    f = h5.H5File(f"{out}.h5")
    steps = int(g["steps"])
    assert sorted(f.keys()) == sorted(["static"] + [f"t{k}" for k in range(steps + 1)])
    np.testing.assert_array_equal(f.read("t0/position"), g["x0"])
    np.testing.assert_array_equal(f.read("static/cell_type").reshape(-1), np.arange(len(g["x0"])) % 3)
    if len(g["links"]):
        np.testing.assert_array_equal(f.read(f"t{steps}/links"), g["links"])


@pytest.mark.gpu
def test_update_functions_between_steps_reproduce_reference(driver, tmp_path):
    """Simulation::run with two UPDATE_FUNC functions (fused per cell on one generator), run_links
    rewiring every link, an INIT_FUNC through init, then three Heun steps: positions, links and the
    DeviceVar counter the functions add to, bit for bit against the reference's run."""
    g, out, r = run_driver(driver, "upd_bg_heun", "upd_bg_heun", tmp_path)
    assert r.returncode == 0, r.stderr
    np.testing.assert_array_equal(np.fromfile(f"{out}.links", np.uint32).reshape(-1, 2), g["links"])
    np.testing.assert_array_equal(np.fromfile(f"{out}.hits", np.int32), g["hits"])
    np.testing.assert_array_equal(np.fromfile(f"{out}.pos", np.float32).reshape(-1, 3), g["pos"])


@pytest.mark.parametrize("name,dims", [("grid_q_3d", 3), ("grid_q_2d", 2)])
def test_host_grid_matches_reference_queries(name, dims, tmp_path):
    """tecs::acceleration::Grid (include/tecs/grid.hpp, the host grid that update functions query) on the
    reference's grid-query fixtures: every query result equal, with the fixtures' stub generator."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    g = dict(np.load(GOLDEN / f"{name}.npz"))
    exe = tmp_path / "grid_host"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
                        str(ROOT / "tests" / "cpp" / "grid_host.cpp"), *link_flags(), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([len(g["x"]), len(g["q"])], np.uint32).tofile(f)
        g["prm"].astype(np.float32).tofile(f)
        g["x"].astype(np.float32).tofile(f)
        g["q"].astype(np.float32).tofile(f)
        g["draws"].astype(np.uint32).tofile(f)
    r = subprocess.run([str(exe), str(dims), str(inp), str(out)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    res = np.fromfile(out, np.int32).reshape(-1, 5)
    for k, key in enumerate(("near1", "near2", "rbins", "rrad", "rfilt")):
        np.testing.assert_array_equal(res[:, k], g[key], err_msg=key)
