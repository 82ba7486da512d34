"""The predefined force functions of the drop-in layer against the reference's.

tests/golden/laws_predefined.npz holds the reference's own functions
(forces/predefined.hpp:60-491: Spring, PiecewiseLinear, PiecewiseQuadratic,
Cubic, Morse, LennardJones, HertzContact) evaluated in float at 233 distances
-- every branch point, the float on either side of it, and a random spread --
by oracle/ref_driver (tests/golden/make_golden.py, LAWS).  tests/cpp/force_laws.cu
evaluates tecs::forces at the same points:

  * on the host (g++): the four polynomial laws bit for bit; Morse,
    LennardJones and HertzContact, which call expf / powf, within 1e-6 of
    the terms they subtract (one libm against another);
  * on a GB300 (nvcc, in a kernel): the polynomial laws bit for bit (the
    library's flags: -fmad=false); the transcendental ones within 4e-6 of
    the terms they subtract (CUDA's expf / powf against libm's; Morse's two
    exponentials cancel near its zero, so its error is relative to them).
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


def term_scale(d):
    """Per distance, the size of the terms each transcendental law subtracts
    (float64, the fixture's parameters): a law's rounding error is relative to
    them, not to their difference, which vanishes at the law's zero."""
    d = d.astype(np.float64)
    dx = d - 1.0
    morse = 2 * 0.25 * (np.exp(-2 * 2.0 * dx) + np.exp(-2.0 * dx))
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        lj = 24 * 0.5 / d * (2 * (0.9 / d) ** 12 + (1.1 / d) ** 6)
    ov = np.maximum(0.6 + 0.7 - d, 0.0)
    e_star = 2.0 * 3.0 / ((1 - 0.09) * 3.0 + (1 - 0.16) * 2.0)
    hertz = 4.0 / 3.0 * e_star * np.sqrt(0.6 * 0.7 / 1.3) * ov ** 1.5
    return {4: morse, 5: lj, 6: hertz}


def compare(mag, vec, g, rtol):
    gm, gv = g["magnitude"], g["vector"]
    np.testing.assert_array_equal(mag[:, POLYNOMIAL], gm[:, POLYNOMIAL])
    np.testing.assert_array_equal(vec[:, POLYNOMIAL], gv[:, POLYNOMIAL])
    terms = term_scale(g["d"])
    for law in TRANSCENDENTAL:
        scale = np.maximum(np.abs(gm[:, law]), terms[law])
        a, b = mag[:, law].astype(np.float64), gm[:, law].astype(np.float64)
        finite = np.isfinite(b)
        np.testing.assert_array_equal(np.isfinite(a), finite)
        np.testing.assert_array_equal(a[~finite], b[~finite])
        with np.errstate(invalid="ignore"):
            assert np.all(np.abs(a - b)[finite] <= rtol * scale[finite]), f"law {law}"
        # each vector component is displacement * F / distance: relative to |F|
        a, b = vec[:, law].astype(np.float64), gv[:, law].astype(np.float64)
        finite = np.isfinite(b)
        # an overflow (LennardJones at a subnormal distance) must overflow alike
        np.testing.assert_array_equal(np.isfinite(a), finite)
        np.testing.assert_array_equal(a[~finite], b[~finite])
        with np.errstate(over="ignore", invalid="ignore"):
            tol = rtol * 2 * (np.abs(g["disp"]) * (scale / np.maximum(g["d"], 1e-30))[:, None])
            ok = (np.abs(a - b) <= np.nan_to_num(tol, nan=0.0)) | (a == b)
        assert np.all(ok[finite]), f"law {law} vector"


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
