"""GB300-native TECS cell-step hot path: Python host front end over the C ABI.

The compute path is the in-tree CUDA library ``_build/libtecs_gb300.so``
(sources in ``csrc/``, C ABI in ``include/tecs_gpu.h``).  This module binds it
with ctypes and mirrors the reference's Simulation / Settings / pair-finder /
integrator vocabulary (include/simulation.hpp:64-668).  There is no CPU
fallback: if the library cannot be loaded every call raises.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from . import build as _build

NAIVE_ALL_PAIRS, BINNED_ALL_PAIRS, NAIVE_GABRIEL, BINNED_GABRIEL, NAIVE_DELAUNAY, DELAUNAY = 0, 1, 2, 3, 4, 5
EULER, HEUN = 0, 1
FORCE_NONE, FORCE_SPRING2R, FORCE_POLARITY = 0, 1, 2

FINDERS = {
    "naive_all_pairs": NAIVE_ALL_PAIRS,
    "binned_all_pairs": BINNED_ALL_PAIRS,
    "naive_gabriel": NAIVE_GABRIEL,
    "binned_gabriel": BINNED_GABRIEL,
    "naive_delaunay": NAIVE_DELAUNAY,
    "delaunay": DELAUNAY,
}
INTEGRATORS = {"euler": EULER, "heun": HEUN}


class TecsError(RuntimeError):
    pass


class SimDesc(ctypes.Structure):
    """Mirror of ``tecs_sim_desc`` (include/tecs_gpu.h)."""

    _fields_ = [
        ("dims", ctypes.c_int),
        ("finder", ctypes.c_int),
        ("symmetric", ctypes.c_int),
        ("cutoff", ctypes.c_float),
        ("gabriel_coefficient", ctypes.c_float),
        ("min_bounds", ctypes.c_float * 3),
        ("max_bounds", ctypes.c_float * 3),
        ("bin_size_scale", ctypes.c_float),
        ("rebuild_every_n", ctypes.c_int),
        ("integrator", ctypes.c_int),
        ("com_fix", ctypes.c_int),
        ("force", ctypes.c_int),
        ("k_rep", ctypes.c_float),
        ("r_rep", ctypes.c_float),
        ("k_adh", ctypes.c_float),
        ("r_adh", ctypes.c_float),
        ("k_pol", ctypes.c_float),
        ("has_polarity", ctypes.c_int),
        ("capacity", ctypes.c_uint),
        ("division_probability", ctypes.c_double),
        ("division_offset", ctypes.c_float),
        ("seed", ctypes.c_uint64),
        ("device", ctypes.c_int),
    ]


_lib = None
_EXPORTS = (
    "tecs_sim_desc_default", "tecs_sim_create", "tecs_sim_destroy", "tecs_sim_upload", "tecs_sim_upload_device",
    "tecs_sim_step", "tecs_sim_synchronize", "tecs_sim_count", "tecs_sim_download", "tecs_sim_evaluate",
    "tecs_sim_stream", "tecs_sim_set_graph", "tecs_sim_kernels_per_step", "tecs_last_error",
    "tecs_sim_set_profiling", "tecs_sim_last_step_profile", "tecs_sim_profile_name", "tecs_sim_set_links",
    "tecs_sim_set_force", "tecs_grid_create", "tecs_grid_destroy", "tecs_grid_rebuild", "tecs_grid_rebuild_device",
    "tecs_grid_query", "tecs_grid_device_view", "tecs_sim_keep_old_velocities", "tecs_sim_old_velocities",
    "tecs_sim_set_old_velocities",
)

GRID_NEAREST, GRID_RANDOM_IN_BINS, GRID_RANDOM_IN_RADIUS = 0, 1, 2


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not _build.LIB.exists() and build_if_missing:
        _build.build()
    if not _build.LIB.exists():
        raise TecsError(f"CUDA library missing: {_build.LIB} (run tecs_gb300.build.build())")
    L = ctypes.CDLL(str(_build.LIB))
    vp, u32p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)
    L.tecs_last_error.restype = ctypes.c_char_p
    L.tecs_sim_desc_default.argtypes = [ctypes.POINTER(SimDesc)]
    L.tecs_sim_create.argtypes = [ctypes.POINTER(SimDesc), ctypes.POINTER(vp)]
    L.tecs_sim_destroy.argtypes = [vp]
    L.tecs_sim_upload.argtypes = [vp, vp, vp, ctypes.c_uint]
    L.tecs_sim_upload_device.argtypes = [vp, vp, vp, ctypes.c_uint]
    L.tecs_sim_step.argtypes = [vp, ctypes.c_double, ctypes.c_int]
    L.tecs_sim_synchronize.argtypes = [vp]
    L.tecs_sim_count.argtypes = [vp, u32p]
    L.tecs_sim_download.argtypes = [vp, vp, vp, u32p]
    L.tecs_sim_evaluate.argtypes = [vp, vp, vp, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    L.tecs_sim_stream.restype = vp
    L.tecs_sim_stream.argtypes = [vp]
    L.tecs_sim_set_graph.argtypes = [vp, ctypes.c_int]
    L.tecs_sim_set_links.argtypes = [vp, vp, ctypes.c_uint, ctypes.c_float]
    L.tecs_sim_set_force.argtypes = [vp, ctypes.c_int] + [ctypes.c_float] * 5
    L.tecs_sim_kernels_per_step.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.tecs_sim_set_profiling.argtypes = [vp, ctypes.c_int]
    L.tecs_sim_last_step_profile.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_int)]
    L.tecs_sim_profile_name.restype = ctypes.c_char_p
    L.tecs_sim_profile_name.argtypes = [vp, ctypes.c_int]
    fp = ctypes.POINTER(ctypes.c_float)
    L.tecs_grid_create.argtypes = [ctypes.c_int, vp, vp, ctypes.c_float, ctypes.c_uint, ctypes.c_int,
                                   ctypes.POINTER(vp)]
    L.tecs_grid_destroy.argtypes = [vp]
    L.tecs_grid_rebuild.argtypes = [vp, vp, ctypes.c_uint]
    L.tecs_grid_rebuild_device.argtypes = [vp, vp, ctypes.c_uint]
    L.tecs_grid_query.argtypes = [vp, ctypes.c_int, vp, ctypes.c_uint, ctypes.c_int, ctypes.c_float, vp, vp, vp]
    L.tecs_grid_device_view.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.tecs_sim_keep_old_velocities.argtypes = [vp, ctypes.c_int]
    L.tecs_sim_old_velocities.argtypes = [vp, vp, u32p]
    L.tecs_sim_set_old_velocities.argtypes = [vp, vp, ctypes.c_uint]
    del fp
    for name in _EXPORTS:
        if name not in ("tecs_last_error", "tecs_sim_stream", "tecs_sim_profile_name"):
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        raise TecsError(load().tecs_last_error().decode())


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


@dataclass
class PairFinderSettings:
    """Binned finders' Settings (binned_gabriel.hpp:20-26, binned_all_pairs.hpp:20-25)."""

    gabriel_coefficient: float = 0.8
    min_bounds: Sequence[float] = (-20.0, -20.0, -20.0)
    max_bounds: Sequence[float] = (20.0, 20.0, 20.0)
    bin_size_scale: float = 1.0
    rebuild_every_n: int = 0


@dataclass
class Spring2R:
    """F(d) = k_rep*max(r_rep-d,0) - k_adh*max(d-r_adh,0); forces::PiecewiseLinear when r_rep == r_adh."""

    k_rep: float = 2.0
    r_rep: float = 0.7
    k_adh: float = 0.5
    r_adh: float = 0.8


@dataclass
class PolaritySpring(Spring2R):
    """Spring2R plus k_pol * (Polarity_::bending_force + bidirectional_polarization_force)."""

    k_pol: float = 0.2


@dataclass
class Division:
    probability: float = 0.0
    offset: float = 0.25


@dataclass
class Settings:
    """Simulation::Settings (include/simulation.hpp:76-98)."""

    agent_count: int
    capacity: int = 0
    cutoff_distance: float = 1.0
    seed: int = 2807
    pair_finder_settings: PairFinderSettings = field(default_factory=PairFinderSettings)


def make_desc(settings: Settings, *, dims: int = 3, pair_finder: str = "binned_gabriel", symmetric: bool = False,
              integrator: str = "heun", com_fixer: Optional[str] = None, force=Spring2R(), polarity: bool = False,
              division: Division = Division(), device: int = 0) -> SimDesc:
    """tecs_sim_desc for a configuration named the reference's way."""
    L = load()
    d = SimDesc()
    _check(L.tecs_sim_desc_default(ctypes.byref(d)))
    pf = settings.pair_finder_settings
    d.dims = dims
    d.finder = FINDERS[pair_finder]
    d.symmetric = int(symmetric)
    d.cutoff = settings.cutoff_distance
    d.gabriel_coefficient = pf.gabriel_coefficient
    for k in range(3):
        d.min_bounds[k] = float(pf.min_bounds[k]) if k < len(pf.min_bounds) else 0.0
        d.max_bounds[k] = float(pf.max_bounds[k]) if k < len(pf.max_bounds) else 0.0
    d.bin_size_scale = pf.bin_size_scale
    d.rebuild_every_n = pf.rebuild_every_n
    d.integrator = INTEGRATORS[integrator]
    d.com_fix = 1 if com_fixer else 0
    if force is None:
        d.force = FORCE_NONE
    else:
        d.force = FORCE_POLARITY if isinstance(force, PolaritySpring) else FORCE_SPRING2R
        d.k_rep, d.r_rep, d.k_adh, d.r_adh = force.k_rep, force.r_rep, force.k_adh, force.r_adh
        d.k_pol = getattr(force, "k_pol", 0.0)
    d.has_polarity = int(polarity)
    d.capacity = max(settings.capacity, settings.agent_count)
    d.division_probability = division.probability
    d.division_offset = division.offset
    d.seed = settings.seed
    d.device = device
    return d


class Simulation:
    """One simulation resident on a GB300: the reference's Simulation<Config>.

    ``pair_finder``: naive_all_pairs | binned_all_pairs | naive_gabriel | binned_gabriel | naive_delaunay |
    delaunay (the Delaunay finder of any capacity, from each cell's star)
    ``integrator``:  euler | heun;  ``com_fixer``: None | "global"
    ``force``: Spring2R | PolaritySpring | None (pair capture only).
    """

    def __init__(self, settings: Settings, *, dims: int = 3, pair_finder: str = "binned_gabriel",
                 symmetric: bool = False, integrator: str = "heun", com_fixer: Optional[str] = None,
                 force=Spring2R(), polarity: bool = False, division: Division = Division(), device: int = 0,
                 graph: bool = True):
        L = load()
        d = make_desc(settings, dims=dims, pair_finder=pair_finder, symmetric=symmetric, integrator=integrator,
                      com_fixer=com_fixer, force=force, polarity=polarity, division=division, device=device)
        self.desc = d
        self.dims = dims
        self.polarity = polarity
        h = ctypes.c_void_p()
        _check(L.tecs_sim_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        if not graph:
            _check(L.tecs_sim_set_graph(h, 0))

    def close(self):
        if getattr(self, "_h", None):
            load().tecs_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state ------------------------------------------------------------
    def set_state(self, positions, polarity=None):
        x = np.ascontiguousarray(positions, dtype=np.float32)
        p = None if polarity is None else np.ascontiguousarray(polarity, dtype=np.float32)
        _check(load().tecs_sim_upload(self._h, _ptr(x), _ptr(p), x.shape[0]))

    def set_links(self, links, strength: float):
        """Links as (a, b) cell-id pairs with the constant-pull link law of strength
        `strength` (examples/intercalation.cpp:65-71); an empty array removes them."""
        lk = np.ascontiguousarray(links, dtype=np.uint32).reshape(-1, 2)
        _check(load().tecs_sim_set_links(self._h, _ptr(lk) if len(lk) else None, lk.shape[0], float(strength)))

    def keep_old_velocities(self, keep: bool = True):
        """Keep the integrator's old velocities (integrators/base.hpp:74): each
        step writes its velocity per cell, and user laws that set drag read
        them."""
        _check(load().tecs_sim_keep_old_velocities(self._h, 1 if keep else 0))

    def get_old_velocities(self):
        v = np.empty((self.desc.capacity, self.dims), np.float32)
        n = ctypes.c_uint()
        _check(load().tecs_sim_old_velocities(self._h, _ptr(v), ctypes.byref(n)))
        return v[: n.value]

    def set_old_velocities(self, v):
        v = np.ascontiguousarray(v, dtype=np.float32).reshape(-1, self.dims)
        _check(load().tecs_sim_set_old_velocities(self._h, _ptr(v) if len(v) else None, v.shape[0]))

    def set_state_device(self, positions_ptr: int, polarity_ptr: Optional[int], n: int):
        _check(load().tecs_sim_upload_device(self._h, ctypes.c_void_p(positions_ptr),
                                             None if polarity_ptr is None else ctypes.c_void_p(polarity_ptr), n))

    def get_agent_count(self) -> int:
        n = ctypes.c_uint()
        _check(load().tecs_sim_count(self._h, ctypes.byref(n)))
        return n.value

    def get_state(self):
        cap = self.desc.capacity
        x = np.empty((cap, self.dims), np.float32)
        p = np.empty((cap, 2), np.float32) if self.polarity else None
        n = ctypes.c_uint()
        _check(load().tecs_sim_download(self._h, _ptr(x), _ptr(p), ctypes.byref(n)))
        return x[: n.value], (p[: n.value] if p is not None else None)

    # -- stepping ---------------------------------------------------------
    def take_step(self, dt: float, n_steps: int = 1):
        _check(load().tecs_sim_step(self._h, float(dt), int(n_steps)))

    def synchronize(self):
        _check(load().tecs_sim_synchronize(self._h))

    @property
    def stream(self) -> int:
        return load().tecs_sim_stream(self._h) or 0

    def kernels_per_step(self) -> int:
        k = ctypes.c_int()
        _check(load().tecs_sim_kernels_per_step(self._h, ctypes.byref(k)))
        return k.value

    # -- profiling --------------------------------------------------------
    def set_profiling(self, enable: bool = True):
        _check(load().tecs_sim_set_profiling(self._h, int(enable)))

    def last_step_profile(self):
        """[(kernel name, ms)] of the most recently completed step, in launch order."""
        buf = (ctypes.c_float * 64)()
        cnt = ctypes.c_int()
        _check(load().tecs_sim_last_step_profile(self._h, buf, 64, ctypes.byref(cnt)))
        out = []
        for k in range(min(cnt.value, 64)):
            name = load().tecs_sim_profile_name(self._h, k)
            out.append(((name or b"?").decode(), float(buf[k])))
        return out

    # -- test hook --------------------------------------------------------
    def evaluate(self, want_pairs: bool = True, pair_capacity: Optional[int] = None):
        """Deltas of one full-step force pass (fresh grid) and the directed id pairs."""
        n = self.get_agent_count()
        dx = np.zeros((max(n, 1), self.dims), np.float32)
        dp = np.zeros((max(n, 1), 2), np.float32) if self.polarity else None
        cnt = ctypes.c_size_t()
        if not want_pairs:
            _check(load().tecs_sim_evaluate(self._h, _ptr(dx), _ptr(dp), None, 0, ctypes.byref(cnt)))
            return dx[:n], (dp[:n] if dp is not None else None), None
        cap = pair_capacity or max(1024, 64 * n)
        while True:
            pairs = np.zeros((cap, 2), np.uint32)
            _check(load().tecs_sim_evaluate(self._h, _ptr(dx), _ptr(dp), _ptr(pairs), cap, ctypes.byref(cnt)))
            if cnt.value <= cap:
                return dx[:n], (dp[:n] if dp is not None else None), pairs[: cnt.value]
            cap = cnt.value


class Grid:
    """A standalone bin grid on the GPU: the reference's acceleration::Grid
    (include/utils/grid.hpp:29-638) -- rebuild over a point set, then nearest
    and random-neighbour queries (tecs_grid_* of the C ABI)."""

    def __init__(self, dims: int, min_bounds, max_bounds, bin_size: float, capacity: int, device: int = 0):
        L = load()
        mn = np.ascontiguousarray(np.asarray(min_bounds, np.float32)[:dims])
        mx = np.ascontiguousarray(np.asarray(max_bounds, np.float32)[:dims])
        h = ctypes.c_void_p()
        _check(L.tecs_grid_create(dims, _ptr(mn), _ptr(mx), float(bin_size), int(capacity), device, ctypes.byref(h)))
        self._h = h
        self.dims = dims
        self.n = 0

    def close(self):
        if getattr(self, "_h", None):
            load().tecs_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rebuild(self, points):
        x = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, self.dims)
        _check(load().tecs_grid_rebuild(self._h, _ptr(x), len(x)))
        self.n = len(x)

    def _query(self, kind, queries, radius_bins=1, radius=0.0, draws=None, eligible=None):
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self.dims)
        out = np.zeros(len(q), np.int32)
        dr = None if draws is None else np.ascontiguousarray(draws, dtype=np.uint32)
        el = None if eligible is None else np.ascontiguousarray(eligible, dtype=np.uint8)
        _check(load().tecs_grid_query(self._h, kind, _ptr(q), len(q), int(radius_bins), float(radius), _ptr(dr),
                                      _ptr(el), _ptr(out)))
        return out

    def nearest(self, queries, radius_bins: int = 1):
        return self._query(GRID_NEAREST, queries, radius_bins=radius_bins)

    def random_in_bins(self, queries, radius_bins: int, draws):
        return self._query(GRID_RANDOM_IN_BINS, queries, radius_bins=radius_bins, draws=draws)

    def random_in_radius(self, queries, radius: float, draws, eligible=None):
        return self._query(GRID_RANDOM_IN_RADIUS, queries, radius=radius, draws=draws, eligible=eligible)


def canonical_pairs(pairs: np.ndarray) -> np.ndarray:
    """Directed pairs sorted by (self, other)."""
    if pairs is None or len(pairs) == 0:
        return np.zeros((0, 2), np.uint32)
    p = np.asarray(pairs, dtype=np.uint32)
    order = np.lexsort((p[:, 1], p[:, 0]))
    return p[order]
