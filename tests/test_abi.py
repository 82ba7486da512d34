"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
entry point that include/tecs_gpu.h declares (no compute calls here)."""
import ctypes
import re
from pathlib import Path

import tecs_gb300 as tg
from tecs_gb300 import build as tb

ROOT = Path(__file__).resolve().parents[1]


def declared(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tecs_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported():
    lib_path = tb.build()
    lib = ctypes.CDLL(str(lib_path))
    names = declared(ROOT / "include" / "tecs_gpu.h")
    assert "tecs_sim_step" in names and "tecs_sim_create" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_desc_layout_matches_header():
    lib = tg.load()
    d = tg.SimDesc()
    assert lib.tecs_sim_desc_default(ctypes.byref(d)) == 0
    # the reference defaults (binned_gabriel.hpp:20-26, simulation.hpp:88-89)
    assert d.dims == 3 and abs(d.gabriel_coefficient - 0.8) < 1e-7
    assert list(d.min_bounds) == [-20.0] * 3 and list(d.max_bounds) == [20.0] * 3
    assert d.bin_size_scale == 1.0 and d.rebuild_every_n == 0 and d.seed == 2807


def test_create_without_gpu_fails_loudly():
    # on a machine without a GPU the product path must raise, never fall back
    from conftest import has_gpu
    if has_gpu():
        return
    try:
        tg.Simulation(tg.Settings(agent_count=10))
    except tg.TecsError as e:
        assert "device" in str(e).lower()
    else:
        raise AssertionError("Simulation() succeeded without a GPU")


def test_null_handles_are_refused_without_touching_a_device():
    # argument checks come before any CUDA call, so they work on a machine without a GPU
    lib = tg.load()
    lib.tecs_last_error.restype = ctypes.c_char_p
    fn = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)(lambda u, c, s: 0)
    lib.tecs_sim_set_pair_law.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    assert lib.tecs_sim_set_pair_law(None, ctypes.cast(fn, ctypes.c_void_p), None) != 0
    assert b"null" in lib.tecs_last_error()
    lib.tecs_sim_set_links.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_float]
    assert lib.tecs_sim_set_links(None, None, 0, 0.0) != 0
    assert b"null" in lib.tecs_last_error()
