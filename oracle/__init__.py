"""ctypes front end of the CPU oracle (test infrastructure only).

The oracle is the CPU result the CUDA path is compared against.  Only the test
suite, ``__graft_entry__.smoke()`` and the benchmark's CPU-baseline leg import
this module; the product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libtecs_oracle.so"
# The timed CPU baseline: the same restatement built the way the reference's
# release build compiles (CMakeLists.txt:195-196: -O3, multiply-add
# contraction left on).  -march=native is left out: host builds here must give
# the same code on the x86 development container and the Arm GPU machine, and
# aarch64's default target already has Advanced SIMD.  Its results are not
# compared bit for bit; only its time is reported.
LIB_TIMING = BUILD / "libtecs_oracle_rel.so"

NAIVE_ALL_PAIRS, BINNED_ALL_PAIRS, NAIVE_GABRIEL, BINNED_GABRIEL, NAIVE_DELAUNAY = 0, 1, 2, 3, 4
FORCE_NONE, FORCE_SPRING2R, FORCE_POLARITY = 0, 1, 2
EULER, HEUN = 0, 1


class Desc(ctypes.Structure):
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
    ]


def reference_root():
    """The TECS reference checkout, or None: $TECS_REFERENCE, else a directory
    named ``reference`` beside this repository.  Only fixture generation and
    the reference-header build read it; nothing on the GPU path does."""
    env = os.environ.get("TECS_REFERENCE")
    cand = Path(env) if env else HERE.parent.parent / "reference"
    return cand if (cand / "include" / "tecs.hpp").exists() else None


def build(force: bool = False, timing: bool = False) -> Path:
    """Compile the C restatement: oracle/_build/libtecs_oracle.so (parity:
    -O2, no multiply-add contraction) or, with timing, the -O3 build of the
    timed CPU baseline."""
    src = HERE / "tecs_oracle.c"
    out = LIB_TIMING if timing else LIB
    if out.exists() and not force and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    BUILD.mkdir(exist_ok=True)
    if timing:
        flags = ["-O3", "-std=gnu11", "-fPIC", "-shared", "-fno-fast-math", "-fopenmp"]
    else:
        flags = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp"]
    tmp = out.with_suffix(".so.tmp")
    subprocess.run(["gcc", *flags, str(src), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, out)
    return out


_libs = {}


def lib(timing: bool = False):
    if timing not in _libs:
        path = build(timing=timing)
        L = ctypes.CDLL(str(path))
        L.tecs_oracle_create.restype = ctypes.c_void_p
        L.tecs_oracle_create.argtypes = [ctypes.POINTER(Desc)]
        L.tecs_oracle_destroy.argtypes = [ctypes.c_void_p]
        L.tecs_oracle_set_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint]
        L.tecs_oracle_count.restype = ctypes.c_uint
        L.tecs_oracle_count.argtypes = [ctypes.c_void_p]
        L.tecs_oracle_get_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.tecs_oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.tecs_oracle_evaluate.restype = ctypes.c_long
        L.tecs_oracle_evaluate.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_long, ctypes.c_int]
        L.tecs_oracle_set_links.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint, ctypes.c_float]
        L.tecs_oracle_hash.restype = ctypes.c_uint64
        L.tecs_oracle_hash.argtypes = [ctypes.c_uint64] * 4
        L.tecs_oracle_last_error.restype = ctypes.c_char_p
        L.tecs_oracle_grid_query.restype = ctypes.c_int
        L.tecs_oracle_grid_query.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_uint,
                                             ctypes.c_void_p, ctypes.c_float] + [ctypes.c_void_p] * 5
        _libs[timing] = L
    return _libs[timing]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """One simulation held by the CPU restatement."""

    def __init__(self, *, dims=3, finder=BINNED_GABRIEL, symmetric=False, cutoff=1.0,
                 gabriel_coefficient=0.8, min_bounds=(-20, -20, -20), max_bounds=(20, 20, 20),
                 bin_size_scale=1.0, rebuild_every_n=0, integrator=HEUN, com_fix=False,
                 force=FORCE_SPRING2R, k_rep=2.0, r_rep=0.7, k_adh=0.5, r_adh=0.8, k_pol=0.0,
                 has_polarity=False, capacity=0, division_probability=0.0, division_offset=0.25,
                 seed=2807, timing=False):
        """timing: hold the simulation in the -O3 build of the timed CPU
        baseline instead of the parity build."""
        self._L = lib(timing)
        d = Desc()
        d.dims, d.finder, d.symmetric = dims, finder, int(symmetric)
        d.cutoff, d.gabriel_coefficient = cutoff, gabriel_coefficient
        for k in range(3):
            d.min_bounds[k] = float(min_bounds[k]) if k < len(min_bounds) else 0.0
            d.max_bounds[k] = float(max_bounds[k]) if k < len(max_bounds) else 0.0
        d.bin_size_scale, d.rebuild_every_n = bin_size_scale, rebuild_every_n
        d.integrator, d.com_fix, d.force = integrator, int(com_fix), force
        d.k_rep, d.r_rep, d.k_adh, d.r_adh, d.k_pol = k_rep, r_rep, k_adh, r_adh, k_pol
        d.has_polarity, d.capacity = int(has_polarity), capacity
        d.division_probability, d.division_offset, d.seed = division_probability, division_offset, seed
        self.desc = d
        self.dims = dims
        self.has_polarity = has_polarity
        self._h = self._L.tecs_oracle_create(ctypes.byref(d))
        if not self._h:
            raise RuntimeError(self._L.tecs_oracle_last_error().decode())

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.tecs_oracle_destroy(h)
            self._h = None

    def set_state(self, positions, polarity=None):
        x = np.ascontiguousarray(positions, dtype=np.float32)
        p = None if polarity is None else np.ascontiguousarray(polarity, dtype=np.float32)
        if self._L.tecs_oracle_set_state(self._h, _ptr(x), _ptr(p), x.shape[0]) != 0:
            raise RuntimeError(self._L.tecs_oracle_last_error().decode())

    def set_links(self, links, strength):
        """(a, b) pairs with the constant-pull link law of strength `strength`."""
        lk = np.ascontiguousarray(links, dtype=np.uint32).reshape(-1, 2)
        if self._L.tecs_oracle_set_links(self._h, _ptr(lk), lk.shape[0], strength) != 0:
            raise RuntimeError(self._L.tecs_oracle_last_error().decode())

    @property
    def count(self):
        return self._L.tecs_oracle_count(self._h)

    def get_state(self):
        n = self.count
        x = np.empty((n, self.dims), np.float32)
        p = np.empty((n, 2), np.float32) if self.has_polarity else None
        self._L.tecs_oracle_get_state(self._h, _ptr(x), _ptr(p))
        return x, p

    def step(self, dt, n_steps=1, threads=1):
        self._L.tecs_oracle_step(self._h, dt, n_steps, threads)

    def evaluate(self, want_pairs=True, threads=1):
        """Deltas of one full-step force pass and the directed pairs in evaluation order."""
        n = self.count
        dx = np.zeros((n, self.dims), np.float32)
        dp = np.zeros((n, 2), np.float32) if self.has_polarity else None
        if not want_pairs:
            self._L.tecs_oracle_evaluate(self._h, _ptr(dx), _ptr(dp), None, 0, threads)
            return dx, dp, None
        cap = max(1024, 64 * n)
        while True:
            pairs = np.zeros((cap, 2), np.uint32)
            cnt = self._L.tecs_oracle_evaluate(self._h, _ptr(dx), _ptr(dp), _ptr(pairs), cap, threads)
            if cnt <= cap:
                return dx, dp, pairs[:cnt]
            cap = cnt


def hash64(seed, step, cell, stream):
    return lib().tecs_oracle_hash(seed, step, cell, stream)


def grid_query(points, min_bounds, max_bounds, bin_size, queries, draws, radius):
    """The reference's acceleration::Grid queries (restated): dict of int32
    arrays near1, near2, rbins, rrad, rfilt (see tecs_oracle_grid_query)."""
    x = np.ascontiguousarray(points, dtype=np.float32)
    q = np.ascontiguousarray(queries, dtype=np.float32)
    dr = np.ascontiguousarray(draws, dtype=np.uint32)
    dims = x.shape[1]
    mn = np.ascontiguousarray(np.asarray(min_bounds, np.float32)[:dims])
    mx = np.ascontiguousarray(np.asarray(max_bounds, np.float32)[:dims])
    out = {k: np.zeros(len(q), np.int32) for k in ("near1", "near2", "rbins", "rrad", "rfilt")}
    rc = lib().tecs_oracle_grid_query(dims, _ptr(x), len(x), _ptr(mn), _ptr(mx), float(bin_size), _ptr(q), len(q),
                                      _ptr(dr), float(radius), *[_ptr(out[k]) for k in
                                                                 ("near1", "near2", "rbins", "rrad", "rfilt")])
    if rc != 0:
        raise RuntimeError(lib().tecs_oracle_last_error().decode())
    return out
