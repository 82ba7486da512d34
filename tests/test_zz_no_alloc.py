"""The allocation-free force pass (tecs_force_pass_noalloc) against tecs_sim_evaluate.

tecs_force_pass_noalloc serves callers that may not allocate device memory
(a host runtime that owns the GPU's memory budget, a serving loop that must not
stall on the allocator): it takes all scratch from a static device array.  This
file runs last in collection order so that, if it fails, every other test has
already run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

RTOL = 1e-5   # the tolerance of the parity tests
ATOL = 1e-6


def _lib():
    L = tg.load()
    L.tecs_force_pass_noalloc.restype = ctypes.c_int
    L.tecs_force_pass_noalloc.argtypes = [ctypes.POINTER(tg.SimDesc), ctypes.c_void_p, ctypes.c_uint,
                                          ctypes.c_void_p, ctypes.c_void_p]
    return L


def _close(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.sqrt(np.mean(b ** 2))
    return bool(np.all(np.abs(a - b) <= RTOL * np.abs(b) + ATOL * scale))


def _reference_deltas(x, finder, mn, mx):
    pf = tg.PairFinderSettings(min_bounds=mn, max_bounds=mx)
    sim = tg.Simulation(tg.Settings(agent_count=len(x), capacity=len(x), pair_finder_settings=pf),
                        pair_finder=finder, force=tg.Spring2R())
    sim.set_state(x)
    dx, _, _ = sim.evaluate(want_pairs=False)
    return sim.desc, dx


@pytest.mark.parametrize("finder", ["binned_gabriel", "binned_all_pairs"])
def test_noalloc_matches_evaluate_twice(finder):
    import torch

    L = _lib()
    # two different inputs in a row: the second call must not see the first's scratch
    inputs = [wl.ball(20000, 21), wl.ball(9000, 22)]
    bounds = wl.bounds_for(inputs[0])
    for x in inputs:
        desc, ref = _reference_deltas(x, finder, *bounds)
        xd = torch.from_numpy(x).cuda()
        out = torch.full((len(x), 3), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = L.tecs_force_pass_noalloc(ctypes.byref(desc), ctypes.c_void_p(xd.data_ptr()), len(x),
                                       ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0, L.tecs_last_error().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert _close(got, ref), float(np.abs(got - ref).max())


def test_noalloc_rejects_oversize():
    L = _lib()
    d = tg.SimDesc()
    L.tecs_sim_desc_default(ctypes.byref(d))
    d.capacity = 1
    rc = L.tecs_force_pass_noalloc(ctypes.byref(d), ctypes.c_void_p(16), 65537, ctypes.c_void_p(16), None)
    assert rc != 0
    assert "allocation-free limit" in L.tecs_last_error().decode()
