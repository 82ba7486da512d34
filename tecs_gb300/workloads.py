"""Seeded synthetic inputs with the shapes of the cell-step benchmark configurations.

No public dataset is involved: every workload is generated here from a seed
(numpy PCG64) and handed identically to the CUDA path and to the oracle.

  ball(n, seed)                     uniform in a ball at density 1 (or radius R)
  sheet(n, seed)                    sphere surface R = sqrt(n/4pi)*0.8, jitter N(0, 0.02)
  outward_polarity(x, seed)         (theta, phi) of the outward normal + N(0, 0.1)
  ensemble(n_sims, seed)            cell counts log-uniform in [500, 200000], per-sim springs
  served_stream(n_req, seed)        Poisson arrivals and request shapes of the served form
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def ball_radius(n: int, density: float = 1.0) -> float:
    return (3.0 * n / (4.0 * math.pi * density)) ** (1.0 / 3.0)


def ball(n: int, seed: int, radius: float | None = None) -> np.ndarray:
    rng = np.random.default_rng(seed)
    R = ball_radius(n) if radius is None else radius
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = R * rng.random(n) ** (1.0 / 3.0)
    return (d * r[:, None]).astype(np.float32)


def disk(n: int, seed: int, density: float = 1.0) -> np.ndarray:
    """n cells uniform in a 2-D disk of the given density."""
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.random(n) * n / (math.pi * density))
    t = rng.random(n) * 2.0 * math.pi
    return np.stack([r * np.cos(t), r * np.sin(t)], axis=1).astype(np.float32)


def sheet_radius(n: int) -> float:
    return math.sqrt(n / (4.0 * math.pi)) * 0.8


def sheet(n: int, seed: int, jitter: float = 0.02) -> np.ndarray:
    rng = np.random.default_rng(seed)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    x = d * sheet_radius(n) + rng.normal(0.0, jitter, (n, 3))
    return x.astype(np.float32)


def outward_polarity(x: np.ndarray, seed: int, noise: float = 0.1) -> np.ndarray:
    """Polarity_(Vector3) convention (types/polarity.hpp:74-77): theta = acos(z/|x|), phi = atan2(y, x)."""
    rng = np.random.default_rng(seed + 7919)
    x64 = x.astype(np.float64)
    r = np.linalg.norm(x64, axis=1)
    th = np.arccos(np.clip(x64[:, 2] / r, -1.0, 1.0)) + rng.normal(0.0, noise, len(x))
    ph = np.arctan2(x64[:, 1], x64[:, 0]) + rng.normal(0.0, noise, len(x))
    return np.stack([th, ph], axis=1).astype(np.float32)


def bounds_for(x: np.ndarray, margin: float = 2.0):
    """Cubic grid bounds covering the cells (the reference default of +-20 would clamp larger domains)."""
    m = float(np.abs(x).max()) + margin
    m = math.ceil(m)
    return (-m, -m, -m), (m, m, m)


@dataclass
class SimSpec:
    n: int
    k_rep: float
    k_adh: float
    gabriel: bool
    seed: int


def ensemble(n_sims: int = 256, seed: int = 2, lo: int = 500, hi: int = 200_000):
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(math.log(lo), math.log(hi), n_sims)).astype(np.int64)
    k_rep = rng.uniform(1.5, 2.5, n_sims)
    k_adh = rng.uniform(0.3, 0.7, n_sims)
    gab = np.zeros(n_sims, bool)
    gab[rng.permutation(n_sims)[: n_sims // 2]] = True
    return [SimSpec(int(ns[k]), float(k_rep[k]), float(k_adh[k]), bool(gab[k]), seed * 100_003 + k)
            for k in range(n_sims)]


@dataclass
class Request:
    arrival_s: float
    n: int
    steps: int
    model: str        # "spring" | "polarity"
    integrator: str   # "euler" | "heun"
    seed: int


def served_stream(n_req: int = 2000, seed: int = 3, rate_hz: float = 20.0, lo: int = 1000, hi: int = 1_000_000,
                  steps_lo: int = 100, steps_hi: int = 1000):
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, n_req))
    ns = np.exp(rng.uniform(math.log(lo), math.log(hi), n_req)).astype(np.int64)
    steps = rng.integers(steps_lo, steps_hi + 1, n_req)
    model = rng.integers(0, 2, n_req)
    integ = rng.integers(0, 2, n_req)
    return [Request(float(t[k]), int(ns[k]), int(steps[k]), ("spring", "polarity")[model[k]],
                    ("euler", "heun")[integ[k]], seed * 1_000_003 + k) for k in range(n_req)]
