"""The polarity pair law on the GB300 against a float64 restatement (GB300).

The law is the reference's Polarity_::bending_force plus
bidirectional_polarization_force (include/types/polarity.hpp:131-198) on top
of the two-radius spring, as the epithelium examples combine them.  Two-cell
configurations -- the axis-aligned polarities of the reference's
tests/test_polarity.cpp and random ones -- are evaluated by the CUDA pass
(both the per-thread path of the naive finder and the block-cooperative path
of the binned Gabriel finder) and by the float64 formulas below; each delta
agrees within |gpu - f64| <= 1e-5 |f64| + 1e-6 s, where s is the larger of
the pair's largest delta and k_pol (the polarity terms are sums of products
of unit-vector components times k_pol, so for configurations where they
cancel to ~0 the float32 rounding of those products, ~1e-7 k_pol, is the
floor).
"""
import math

import numpy as np
import pytest

import tecs_gb300 as tg

pytestmark = pytest.mark.gpu

K_REP, R_REP, K_ADH, R_ADH, K_POL = 2.0, 0.7, 0.5, 0.8, 0.2


def to_vec(p):
    th, ph = p
    return np.array([math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)])


def unidirectional(s, o):
    r0 = math.cos(s[0]) * math.sin(o[0]) * math.cos(s[1] - o[1]) - math.sin(s[0]) * math.cos(o[0])
    st = math.sin(s[0])
    r1 = -math.sin(o[0]) * math.sin(s[1] - o[1]) / st if abs(st) > 1.1920929e-07 else 0.0
    return np.array([r0, r1])


def pol_dot(s, o):
    return math.sin(s[0]) * math.sin(o[0]) * math.cos(s[1] - o[1]) + math.cos(s[0]) * math.cos(o[0])


def pair_f64(xi, xj, pi, pj):
    """Deltas (position, polarity) the pair (self i, other j) adds to cell i."""
    disp = np.asarray(xi, np.float64) - np.asarray(xj, np.float64)
    dist = float(np.linalg.norm(disp))
    F = K_REP * max(R_REP - dist, 0.0) - K_ADH * max(dist - R_ADH, 0.0)
    dx = disp * F / dist
    tv, ov = to_vec(pi), to_vec(pj)
    prod_i = float(tv @ disp) / dist
    prod_j = float(ov @ disp) / dist
    bend = -prod_i / dist * tv + prod_i ** 2 / dist ** 2 * disp - prod_j / dist * ov + prod_j ** 2 / dist ** 2 * disp
    dpol = (math.acos(min(1.0, max(-1.0, disp[2] / dist))), math.atan2(disp[1], disp[0]))
    bend_pol = -prod_i * unidirectional(pi, dpol)
    align = pol_dot(pi, pj) * unidirectional(pi, pj)
    return dx + K_POL * bend, K_POL * (bend_pol + align)


HALF_PI = math.pi / 2
AXES = {"x": (HALF_PI, 0.0), "y": (HALF_PI, HALF_PI), "z": (0.0, 0.0)}


def cases():
    rng = np.random.default_rng(17)
    out = []
    # the reference test's axis polarities, cells apart along each axis
    for a in AXES:
        for b in AXES:
            for axis in range(3):
                d = np.zeros(3)
                d[axis] = 0.75
                out.append((np.zeros(3), d, AXES[a], AXES[b]))
    for _ in range(24):
        d = rng.normal(size=3)
        d *= rng.uniform(0.3, 0.95) / np.linalg.norm(d)
        out.append((rng.normal(size=3), None, (float(rng.uniform(0.1, 3.0)), float(rng.uniform(-3, 3))),
                    (float(rng.uniform(0.1, 3.0)), float(rng.uniform(-3, 3)))))
        out[-1] = (out[-1][0], out[-1][0] + d, out[-1][2], out[-1][3])
    return out


@pytest.mark.parametrize("finder", ["naive_all_pairs", "binned_gabriel"])
def test_two_cell_polarity_law_matches_f64(finder):
    worst = 0.0
    for x0, x1, p0, p1 in cases():
        x = np.array([x0, x1], np.float32)
        p = np.array([p0, p1], np.float32)
        mn, mx = tg_bounds(x)
        s = tg.Simulation(tg.Settings(agent_count=2, capacity=2, pair_finder_settings=tg.PairFinderSettings(
            min_bounds=mn, max_bounds=mx)), pair_finder=finder, integrator="euler",
            force=tg.PolaritySpring(k_rep=K_REP, r_rep=R_REP, k_adh=K_ADH, r_adh=R_ADH, k_pol=K_POL), polarity=True)
        s.set_state(x, p)
        dx, dp, pairs = s.evaluate()
        assert len(pairs) == 2
        # the float64 law on the float32 inputs the kernel saw
        xf, pf = x.astype(np.float64), p.astype(np.float64)
        for i, j in ((0, 1), (1, 0)):
            ex, ep = pair_f64(xf[i], xf[j], tuple(pf[i]), tuple(pf[j]))
            scale = max(np.abs(ex).max(), np.abs(ep).max(), K_POL)
            for got, want in ((dx[i], ex), (dp[i], ep)):
                err = np.abs(got.astype(np.float64) - want)
                assert (err <= 1e-5 * np.abs(want) + 1e-6 * scale).all(), (finder, x0, x1, p0, p1, got, want)
                worst = max(worst, float((err / scale).max()))
        s.close()
    assert worst < 1e-6  # relative to the scale above


def test_orthogonal_and_parallel_alignment_known_answers():
    # dot(p, p) = 1 and dot(pX, pY) = 0 (tests/test_polarity.cpp:52-72): the
    # alignment term vanishes for orthogonal polarities and the bending term
    # vanishes for polarities perpendicular to the displacement
    x = np.array([[0, 0, 0], [0, 0, 0.75]], np.float32)  # displacement along z
    p = np.array([AXES["x"], AXES["y"]], np.float32)      # both perpendicular to it, mutually orthogonal
    mn, mx = tg_bounds(x)
    s = tg.Simulation(tg.Settings(agent_count=2, capacity=2, pair_finder_settings=tg.PairFinderSettings(
        min_bounds=mn, max_bounds=mx)), pair_finder="naive_all_pairs", integrator="euler",
        force=tg.PolaritySpring(k_rep=K_REP, r_rep=R_REP, k_adh=K_ADH, r_adh=R_ADH, k_pol=K_POL), polarity=True)
    s.set_state(x, p)
    dx, dp, _ = s.evaluate()
    # d = 0.75 lies between r_rep and r_adh: no spring force either
    np.testing.assert_allclose(dx, 0.0, atol=1e-6)
    np.testing.assert_allclose(dp, 0.0, atol=1e-6)
    s.close()


def tg_bounds(x):
    m = float(np.ceil(np.abs(x).max() + 2.0))
    return (-m, -m, -m), (m, m, m)
