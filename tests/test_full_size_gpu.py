"""The benchmark configurations compared with the oracle at their stated sizes (GB300).

  * epithelial sheet, 100,000 cells with polarity (the bench's sheet workload):
    one pass pair for pair, five Heun steps within the polarity tolerance, and
    500 steps by trajectory statistics;
  * spheroid, 1,000,000 cells (the bench's headline workload): ten Heun steps
    with the COM fix and division at 1e-4 -- agent count exact, positions
    within tolerance -- and the 4,000,000-cell point pair for pair and bit for
    bit in one pass;
  * the error of each result against a float64 recompute of the same pairs:
    the spring deltas of one pass and the one-step displacement of an Euler
    step with the COM fix (position delta minus the capacity mean), both at
    1,000,000 cells.  The bound written here is the parity tolerance, and the
    CUDA result's error must equal the oracle's (they are the same bits) or,
    with the COM sum, stay within twice it.
"""
import numpy as np
import pytest

import oracle
import tecs_gb300 as tg
from tecs_gb300 import workloads as wl

from test_long_run_statistics_gpu import mean_neighbours, polarity_order, radius_of_gyration
from test_parity_gpu import close, make_pair

pytestmark = pytest.mark.gpu

RTOL = 1e-5
ATOL = 1e-6


def sheet_100k():
    x = wl.sheet(100_000, 1)
    p = wl.outward_polarity(x, 1)
    return x, p, wl.bounds_for(x, margin=2.0)


def spheroid(n):
    x = wl.ball(n, 1)
    return x, wl.bounds_for(x, margin=2.0)


def spring_f64(x, pairs, k_rep=2.0, r_rep=0.7, k_adh=0.5, r_adh=0.8):
    """Per-cell sum over the directed pairs (self, other) of disp * F(d) / d in float64."""
    x = x.astype(np.float64)
    i, j = pairs[:, 0].astype(np.int64), pairs[:, 1].astype(np.int64)
    disp = x[i] - x[j]
    d = np.sqrt((disp ** 2).sum(1))
    F = k_rep * np.maximum(r_rep - d, 0.0) - k_adh * np.maximum(d - r_adh, 0.0)
    f = disp * (F / np.where(d > 0, d, 1.0))[:, None]
    out = np.zeros_like(x)
    for k in range(x.shape[1]):
        out[:, k] = np.bincount(i, weights=f[:, k], minlength=len(x))
    return out


def unit(p):
    th, ph = p[:, 0].astype(np.float64), p[:, 1].astype(np.float64)
    return np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)


def rel_error(got, ref):
    """max over components of |got - ref| / (|ref| + 1e-6 rms(ref)) and the fraction above RTOL."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = np.sqrt(np.mean(ref ** 2))
    e = np.abs(got - ref) / (np.abs(ref) + (ATOL / RTOL) * scale)
    return float(e.max()), float(np.mean(e > RTOL))


def test_sheet_100k_pass_and_heun_steps():
    x, p, bounds = sheet_100k()
    g, c = make_pair(x, finder="binned_gabriel", force="polarity", pol=p, bounds=bounds)
    dg, pg, pairs_g = g.evaluate()
    dc, pc, pairs_c = c.evaluate(threads=0)
    np.testing.assert_array_equal(tg.canonical_pairs(pairs_g), tg.canonical_pairs(pairs_c))
    ok, err, nbad = close(dg, dc)
    assert ok, ("position deltas", err, nbad)
    ok, err, nbad = close(pg, pc)
    assert ok, ("polarity deltas", err, nbad)
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun", force="polarity", pol=p, bounds=bounds)
    g.take_step(0.05, 5)
    c.step(0.05, 5, 0)
    xg, qg = g.get_state()
    xc, qc = c.get_state()
    ok, err, nbad = close(xg, xc, atol=1e-5)
    assert ok, ("positions", err, nbad)
    # polarities as unit vectors: the angle phi of a polarity near a pole
    # (theta ~ 0) is ill-conditioned, its direction is not.  Five steps of
    # the law's sin/cos/acos (CUDA's against libm's, each within a few ulp)
    # move a few of the 100,000 directions by more than 1e-5: every direction
    # within 5e-5 rad of the oracle's, and at most 1 in 10,000 beyond 1e-5
    ug, uc = unit(qg), unit(qc)
    angle = np.linalg.norm(ug - uc, axis=1)
    assert angle.max() <= 5e-5, ("polarities", float(angle.max()))
    assert np.mean(angle > 1e-5) <= 1e-4, ("polarities beyond 1e-5", int(np.sum(angle > 1e-5)))


def test_sheet_100k_500_steps_statistics():
    # the configuration's full run length; statistics every 100 steps with the
    # tolerances of the long-run tests
    x, p, bounds = sheet_100k()
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun", force="polarity", pol=p, bounds=bounds)
    for _ in range(5):
        g.take_step(0.05, 100)
        c.step(0.05, 100, 0)
        xg, qg = g.get_state()
        xc, qc = c.get_state()
        ng, nc = mean_neighbours(xg), mean_neighbours(xc)
        assert abs(ng - nc) <= 1e-3 * nc, (ng, nc)
        rg, rc_ = radius_of_gyration(xg), radius_of_gyration(xc)
        assert abs(rg - rc_) <= 1e-4 * rc_, (rg, rc_)
        og, oc = polarity_order(qg), polarity_order(qc)
        assert abs(og - oc) <= 1e-3, (og, oc)


def test_spheroid_1m_heun_com_division_ten_steps():
    n = 1_000_000
    x, bounds = spheroid(n)
    cap = 1_050_000
    g, c = make_pair(x, finder="binned_gabriel", integrator="heun", com=True, division=1e-4, capacity=cap,
                     bounds=bounds)
    g.take_step(0.05, 10)
    c.step(0.05, 10, 0)
    assert g.get_agent_count() == c.count > n
    xg, _ = g.get_state()
    xc, _ = c.get_state()
    ok, err, nbad = close(xg, xc, atol=1e-5)
    assert ok, (err, nbad)
    ng, nc = mean_neighbours(xg), mean_neighbours(xc)
    assert abs(ng - nc) <= 1e-3 * nc, (ng, nc)


def test_spheroid_4m_pass_pairs_and_deltas_bit_exact():
    x, bounds = spheroid(4_000_000)
    g, c = make_pair(x, finder="binned_gabriel", com=True, capacity=4_200_000, bounds=bounds)
    dg, _, pg = g.evaluate()
    dc, _, pc = c.evaluate(threads=0)
    np.testing.assert_array_equal(tg.canonical_pairs(pg), tg.canonical_pairs(pc))
    np.testing.assert_array_equal(dg, dc)


def test_spheroid_1m_errors_against_float64():
    n = 1_000_000
    x, bounds = spheroid(n)
    cap = 1_050_000
    # (1) the spring deltas of one full-step pass
    g, c = make_pair(x, finder="binned_gabriel", capacity=cap, bounds=bounds)
    dg, _, pairs = g.evaluate()
    dc, _, _ = c.evaluate(want_pairs=False, threads=0)
    d64 = spring_f64(x, pairs)
    eg, fg = rel_error(dg, d64)
    ec, fc = rel_error(dc, d64)
    print(f"\nspring deltas vs float64: CUDA max rel {eg:.3e} (above 1e-5: {fg:.2e}), oracle {ec:.3e}")
    assert eg == ec
    assert eg <= RTOL, eg
    # (2) one Euler step with the COM fix: x1 - x0 = (d - c) dt with c the
    # capacity mean (com_fixers.hpp:31-43, euler.hpp:49-69)
    dt = 0.05
    g, c = make_pair(x, finder="binned_gabriel", integrator="euler", com=True, capacity=cap, bounds=bounds)
    g.take_step(dt, 1)
    c.step(dt, 1, 0)
    x1g, _ = g.get_state()
    x1c, _ = c.get_state()
    c64 = d64.sum(0) / cap
    disp64 = (d64 - c64) * dt
    eg, fg = rel_error(x1g.astype(np.float64) - x, disp64)
    ec, fc = rel_error(x1c.astype(np.float64) - x, disp64)
    print(f"one-step displacement vs float64: CUDA max rel {eg:.3e} (above 1e-5: {fg:.2e}), oracle {ec:.3e}")
    # the displacement is formed from float32 positions (|x| up to ~64), so its
    # rounding is relative to |x|, not to the displacement: stated, and bounded
    # by the oracle's own error
    assert eg <= 2.0 * ec + 1e-12, (eg, ec)
