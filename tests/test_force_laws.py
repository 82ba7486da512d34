"""The predefined force functions of the drop-in layer against the reference's.

tests/golden/laws_predefined.npz holds the reference's own functions
(forces/predefined.hpp:60-491: Spring, PiecewiseLinear, PiecewiseQuadratic,
Cubic, Morse, LennardJones, HertzContact) evaluated in float at 233 distances
-- every branch point, the float on either side of it, and a random spread --
by oracle/ref_driver (tests/golden/make_golden.py, LAWS).  tests/cpp/force_laws.cu
evaluates tecs::forces at the same points:

  * on the host (g++): the four polynomial laws bit for bit; Morse,
    LennardJones and HertzContact, which call expf / powf, within 1e-6
    relative (one libm against another);
  * on a GB300 (nvcc, in a kernel): the polynomial laws bit for bit (the
    library's flags: -fmad=false); the transcendental ones within 4e-6
    relative of the magnitude (CUDA's expf / powf against libm's).
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
SOURCE = Path(__file__).resolve().parent / "cpp" / "force_laws.cu"
POLYNOMIAL = [0, 1, 2, 3]
TRANSCENDENTAL = [4, 5, 6]


def write_input(path, g):
    with open(path, "wb") as f:
        np.array([len(g["d"])], np.uint32).tofile(f)
        g["d"].astype(np.float32).tofile(f)
        g["disp"].astype(np.float32).tofile(f)


def run(exe, g, tmp_path):
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    write_input(inp, g)
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    res = np.fromfile(out, np.float32).reshape(len(g["d"]), 28)
    return res[:, :7], res[:, 7:].reshape(len(g["d"]), 7, 3)


def compare(mag, vec, g, rtol):
    gm, gv = g["magnitude"], g["vector"]
    np.testing.assert_array_equal(mag[:, POLYNOMIAL], gm[:, POLYNOMIAL])
    np.testing.assert_array_equal(vec[:, POLYNOMIAL], gv[:, POLYNOMIAL])
    for law in TRANSCENDENTAL:
        scale = np.abs(gm[:, law])
        np.testing.assert_allclose(mag[:, law], gm[:, law], rtol=rtol, atol=0, err_msg=f"law {law}")
        # each vector component is displacement * F / distance: relative to |F|
        a, b = vec[:, law].astype(np.float64), gv[:, law].astype(np.float64)
        finite = np.isfinite(b)
        # an overflow (LennardJones at a subnormal distance) must overflow alike
        np.testing.assert_array_equal(np.isfinite(a), finite)
        np.testing.assert_array_equal(a[~finite], b[~finite])
        with np.errstate(over="ignore", invalid="ignore"):
            tol = rtol * 2 * (np.abs(g["disp"]) * (scale / np.maximum(g["d"], 1e-30))[:, None]) + 1e-30
        assert np.all(np.abs(a - b)[finite] <= tol[finite]), f"law {law} vector"


def test_fixture_covers_branch_points():
    g = dict(np.load(GOLDEN / "laws_predefined.npz"))
    assert g["magnitude"].shape == (len(g["d"]), 7)
    # each law takes its zero, repulsive and adhesive branches somewhere in the table
    for law in range(7):
        m = g["magnitude"][:, law]
        assert (m > 0).any(), law
    for law in (0, 1, 2, 3, 4, 5):
        assert (g["magnitude"][:, law] < 0).any(), law
    assert (g["magnitude"][:, 6] == 0).any()
    # distance 0 gives the zero vector
    assert np.all(g["vector"][g["d"] == 0] == 0)


def test_host_functions_match_reference(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    g = dict(np.load(GOLDEN / "laws_predefined.npz"))
    exe = tmp_path / "force_laws"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-Wall", "-Wextra", "-Werror", "-x", "c++",
                        f"-I{ROOT / 'include'}", str(SOURCE), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    mag, vec = run(exe, g, tmp_path)
    compare(mag, vec, g, 1e-6)


@pytest.mark.gpu
def test_device_functions_match_reference(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    g = dict(np.load(GOLDEN / "laws_predefined.npz"))
    exe = tmp_path / "force_laws_gpu"
    r = subprocess.run([nvcc, "-std=c++20", "-O2", "-fmad=false", "-gencode", "arch=compute_103a,code=sm_103a",
                        f"-I{ROOT / 'include'}", str(SOURCE), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    mag, vec = run(exe, g, tmp_path)
    compare(mag, vec, g, 4e-6)
