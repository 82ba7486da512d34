"""The allocation-free force pass (tecs_force_pass_noalloc) against tecs_sim_evaluate.

tecs_force_pass_noalloc serves callers that may not allocate device memory
(a host runtime that owns the GPU's memory budget, a serving loop that must not
stall on the allocator): it takes all scratch from a static device array.  It
runs the same rebuild and pass kernels as tecs_sim_evaluate, so its deltas
must be the same bits.  This file runs last in collection order so that, if it
fails, every other test has already run; it also passes alone in a fresh
process.
"""
import ctypes

import numpy as np
import pytest

import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _lib():
    L = tg.load()
    L.tecs_force_pass_noalloc.restype = ctypes.c_int
    L.tecs_force_pass_noalloc.argtypes = [ctypes.POINTER(tg.SimDesc), ctypes.c_void_p, ctypes.c_uint,
                                          ctypes.c_void_p, ctypes.c_void_p]
    return L


def _reference_deltas(x, finder, mn, mx, dims):
    pf = tg.PairFinderSettings(min_bounds=mn, max_bounds=mx)
    sim = tg.Simulation(tg.Settings(agent_count=len(x), capacity=len(x), pair_finder_settings=pf), dims=dims,
                        pair_finder=finder, force=tg.Spring2R())
    sim.set_state(x)
    dx, _, _ = sim.evaluate(want_pairs=False)
    sim.close()
    return sim.desc, dx


def _noalloc(L, desc, x):
    import torch

    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    out = torch.full(x.shape, float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = L.tecs_force_pass_noalloc(ctypes.byref(desc), ctypes.c_void_p(xd.data_ptr()), len(x),
                                   ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 0, L.tecs_last_error().decode()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _disk(n, seed):
    rng = np.random.default_rng(seed)
    r = np.sqrt(n / np.pi) * np.sqrt(rng.random(n))
    a = rng.random(n) * 2 * np.pi
    return np.stack([r * np.cos(a), r * np.sin(a)], axis=1).astype(np.float32)


@pytest.mark.parametrize("finder", ["binned_gabriel", "binned_all_pairs"])
def test_noalloc_matches_evaluate_twice(finder):
    L = _lib()
    # two different inputs in a row: the second call must not see the first's scratch
    inputs = [wl.ball(20000, 21), wl.ball(9000, 22)]
    bounds = wl.bounds_for(inputs[0])
    for x in inputs:
        desc, ref = _reference_deltas(x, finder, *bounds, dims=3)
        got = _noalloc(L, desc, x)
        assert np.array_equal(got, ref), float(np.abs(got - ref).max())


def test_noalloc_two_dimensions():
    L = _lib()
    for seed in (23, 24):
        x = _disk(6000, seed)
        m = float(np.ceil(np.abs(x).max() + 2))
        desc, ref = _reference_deltas(x, "binned_gabriel", (-m, -m, 0.0), (m, m, 0.0), dims=2)
        got = _noalloc(L, desc, x)
        assert np.array_equal(got, ref), float(np.abs(got - ref).max())


def test_noalloc_sparse_grid():
    # bins > 4 x cells (the evaluate path then forms the scan's chunk totals
    # while counting) but within the allocation-free bin limit
    L = _lib()
    x = wl.ball(3000, 25)
    m = 28.0  # 56^3 = 175,616 bins for 3,000 cells
    assert (2 * m) ** 3 > 4 * len(x) and (2 * m) ** 3 <= 262144
    for _ in range(2):
        desc, ref = _reference_deltas(x, "binned_gabriel", (-m, -m, -m), (m, m, m), dims=3)
        got = _noalloc(L, desc, x)
        assert np.array_equal(got, ref), float(np.abs(got - ref).max())


def test_noalloc_rejects_oversize():
    L = _lib()
    d = tg.SimDesc()
    L.tecs_sim_desc_default(ctypes.byref(d))
    d.capacity = 1
    rc = L.tecs_force_pass_noalloc(ctypes.byref(d), ctypes.c_void_p(16), 65537, ctypes.c_void_p(16), None)
    assert rc != 0
    assert "allocation-free limit" in L.tecs_last_error().decode()
