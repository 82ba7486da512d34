"""State transfers through the C ABI: page-locked host buffers are read and
written by kernels directly (tecs_sim_upload / tecs_sim_download); any other
host memory goes through a staged copy.  Both routes must give the same
simulation, bit for bit, including polarity, division growth and destination
buffers that are not 16-byte aligned.
"""
import ctypes

import numpy as np
import pytest

import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def make(x, pol, capacity):
    mn, mx = wl.bounds_for(x)
    return tg.Simulation(tg.Settings(agent_count=len(x), capacity=capacity,
                                     pair_finder_settings=tg.PairFinderSettings(min_bounds=mn, max_bounds=mx)),
                         pair_finder="binned_gabriel", integrator="heun", com_fixer="global",
                         force=tg.PolaritySpring(k_pol=0.2) if pol else tg.Spring2R(), polarity=pol,
                         division=tg.Division(probability=2e-3))


def pinned(shape, offset_floats=0):
    """A page-locked float32 buffer of `shape`, starting `offset_floats` into its allocation."""
    n = int(np.prod(shape))
    t = torch.zeros(n + offset_floats, dtype=torch.float32, pin_memory=True)
    return t, t[offset_floats:].view(*shape)


def upload_pinned(sim, x, p):
    L = tg.load()
    _, hx = pinned(x.shape)
    hx.numpy()[:] = x
    hp = None
    if p is not None:
        _, hp = pinned(p.shape)
        hp.numpy()[:] = p
    tg._check(L.tecs_sim_upload(sim._h, ctypes.c_void_p(hx.data_ptr()),
                                None if hp is None else ctypes.c_void_p(hp.data_ptr()), len(x)))


def download_pinned(sim, offset_floats):
    L = tg.load()
    cap = sim.desc.capacity
    keep_x, hx = pinned((cap, sim.dims), offset_floats)
    keep_p, hp = pinned((cap, 2), offset_floats) if sim.polarity else (None, None)
    n = ctypes.c_uint()
    tg._check(L.tecs_sim_download(sim._h, ctypes.c_void_p(hx.data_ptr()),
                                  None if hp is None else ctypes.c_void_p(hp.data_ptr()), ctypes.byref(n)))
    x = hx.numpy()[: n.value].copy()
    p = hp.numpy()[: n.value].copy() if hp is not None else None
    return x, p


@pytest.mark.parametrize("pol", [False, True])
@pytest.mark.parametrize("offset", [0, 1, 3])
def test_pinned_and_pageable_transfers_give_the_same_run(pol, offset):
    x = wl.sheet(3000, 5) if pol else wl.ball(5000, 4)
    p = wl.outward_polarity(x, 5) if pol else None
    cap = int(len(x) * 1.2)
    a, b = make(x, pol, cap), make(x, pol, cap)
    a.set_state(x, p)          # numpy buffers: staged copies
    upload_pinned(b, x, p)     # page-locked buffers: read by the upload kernel
    # a round trip without steps returns the input
    xb, pb = download_pinned(b, offset)
    np.testing.assert_array_equal(xb, x)
    if pol:
        np.testing.assert_array_equal(pb, p)
    for _ in range(3):
        a.take_step(0.05, 10)
        b.take_step(0.05, 10)
        xa, pa = a.get_state()
        xb, pb = download_pinned(b, offset)
        assert len(xa) == len(xb)
        np.testing.assert_array_equal(xa, xb)
        if pol:
            np.testing.assert_array_equal(pa, pb)
        # continue both from the downloaded state, through the other route
        a.set_state(xb, pb)
        upload_pinned(b, xa, pa)
    assert a.get_agent_count() > len(x)  # division grew both the same way
