"""Many simulations on one GB300: ctypes front end of the tecs_engine C ABI.

An Engine holds every resident simulation in one set of device arrays and
advances all of them with one CUDA-graph step (include/tecs_gpu.h,
tecs_engine_*).  Each simulation is described like a single one (make_desc)
and evolves exactly as a tecs_gb300.Simulation of it would.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import SimDesc, TecsError, _check, _ptr, load


class EngineDesc(ctypes.Structure):
    _fields_ = [("cell_capacity", ctypes.c_uint), ("bin_capacity", ctypes.c_uint), ("max_sims", ctypes.c_uint),
                ("device", ctypes.c_int)]


_bound = False


def _lib():
    global _bound
    L = load()
    if _bound:
        return L
    vp, up = ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)
    L.tecs_engine_desc_default.argtypes = [ctypes.POINTER(EngineDesc)]
    L.tecs_engine_create.argtypes = [ctypes.POINTER(EngineDesc), ctypes.POINTER(vp)]
    L.tecs_engine_destroy.argtypes = [vp]
    L.tecs_engine_bins_needed.argtypes = [ctypes.POINTER(SimDesc), up]
    L.tecs_engine_free.argtypes = [vp, up, up]
    L.tecs_engine_set_pass_threads.argtypes = [vp, ctypes.c_uint]
    L.tecs_engine_add.argtypes = [vp, ctypes.POINTER(SimDesc), vp, vp, ctypes.c_uint, ctypes.POINTER(ctypes.c_int)]
    L.tecs_engine_remove.argtypes = [vp, ctypes.c_int]
    L.tecs_engine_step.argtypes = [vp, ctypes.c_double, ctypes.c_int]
    L.tecs_engine_synchronize.argtypes = [vp]
    L.tecs_engine_count.argtypes = [vp, up, up]
    L.tecs_engine_download.argtypes = [vp, ctypes.c_int, vp, vp, up]
    L.tecs_engine_snapshot_async.argtypes = [vp, ctypes.c_int, vp, vp, ctypes.c_uint, ctypes.POINTER(vp)]
    L.tecs_engine_event_query.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.tecs_engine_event_destroy.argtypes = [vp]
    L.tecs_engine_kernels_per_step.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.tecs_engine_stream.restype = vp
    L.tecs_engine_stream.argtypes = [vp]
    for name in ("tecs_engine_desc_default", "tecs_engine_create", "tecs_engine_destroy", "tecs_engine_bins_needed",
                 "tecs_engine_free", "tecs_engine_add", "tecs_engine_remove", "tecs_engine_step",
                 "tecs_engine_synchronize", "tecs_engine_count", "tecs_engine_download", "tecs_engine_snapshot_async",
                 "tecs_engine_event_query", "tecs_engine_event_destroy", "tecs_engine_kernels_per_step",
                 "tecs_engine_set_pass_threads"):
        getattr(L, name).restype = ctypes.c_int
    _bound = True
    return L


def bins_needed(desc: SimDesc) -> int:
    nb = ctypes.c_uint()
    _check(_lib().tecs_engine_bins_needed(ctypes.byref(desc), ctypes.byref(nb)))
    return nb.value


class Engine:
    def __init__(self, cell_capacity: int, bin_capacity: int, max_sims: int = 1024, device: int = 0):
        L = _lib()
        d = EngineDesc()
        _check(L.tecs_engine_desc_default(ctypes.byref(d)))
        d.cell_capacity, d.bin_capacity, d.max_sims, d.device = cell_capacity, bin_capacity, max_sims, device
        h = ctypes.c_void_p()
        _check(L.tecs_engine_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self.desc = d
        self.sims = {}

    def close(self):
        if getattr(self, "_h", None):
            _lib().tecs_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_pass_threads(self, threads: int):
        """Threads per block of the force passes: 64, 96 or 128 (results do not depend on it)."""
        _check(_lib().tecs_engine_set_pass_threads(self._h, int(threads)))

    def free(self):
        c, b = ctypes.c_uint(), ctypes.c_uint()
        _check(_lib().tecs_engine_free(self._h, ctypes.byref(c), ctypes.byref(b)))
        return c.value, b.value

    def add(self, desc: SimDesc, positions, polarity=None) -> int:
        x = np.ascontiguousarray(positions, dtype=np.float32)
        p = None if polarity is None else np.ascontiguousarray(polarity, dtype=np.float32)
        slot = ctypes.c_int()
        _check(_lib().tecs_engine_add(self._h, ctypes.byref(desc), _ptr(x), _ptr(p), x.shape[0], ctypes.byref(slot)))
        self.sims[slot.value] = (x.shape[0], bool(desc.has_polarity))
        return slot.value

    def remove(self, slot: int):
        _check(_lib().tecs_engine_remove(self._h, slot))
        self.sims.pop(slot, None)

    def step(self, dt: float, n_steps: int = 1):
        _check(_lib().tecs_engine_step(self._h, float(dt), int(n_steps)))

    def synchronize(self):
        _check(_lib().tecs_engine_synchronize(self._h))

    def count(self):
        c, s = ctypes.c_uint(), ctypes.c_uint()
        _check(_lib().tecs_engine_count(self._h, ctypes.byref(c), ctypes.byref(s)))
        return c.value, s.value

    def download(self, slot: int):
        n, pol = self.sims[slot]
        x = np.empty((max(n, 1), 3), np.float32)
        p = np.empty((max(n, 1), 2), np.float32) if pol else None
        nn = ctypes.c_uint()
        _check(_lib().tecs_engine_download(self._h, slot, _ptr(x), _ptr(p), ctypes.byref(nn)))
        return x[:n], (p[:n] if p is not None else None)

    def snapshot_async(self, slot: int, pinned_positions_ptr: int, pinned_polarity_ptr: Optional[int],
                       stage_offset: int = 0):
        ev = ctypes.c_void_p()
        _check(_lib().tecs_engine_snapshot_async(self._h, slot, ctypes.c_void_p(pinned_positions_ptr),
                                                 None if pinned_polarity_ptr is None else
                                                 ctypes.c_void_p(pinned_polarity_ptr),
                                                 stage_offset, ctypes.byref(ev)))
        return ev

    @staticmethod
    def event_ready(ev) -> bool:
        r = ctypes.c_int()
        _check(_lib().tecs_engine_event_query(ev, ctypes.byref(r)))
        return bool(r.value)

    @staticmethod
    def event_destroy(ev):
        _lib().tecs_engine_event_destroy(ev)

    def kernels_per_step(self) -> int:
        k = ctypes.c_int()
        _check(_lib().tecs_engine_kernels_per_step(self._h, ctypes.byref(k)))
        return k.value

    @property
    def stream(self) -> int:
        return _lib().tecs_engine_stream(self._h) or 0
