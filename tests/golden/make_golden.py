#!/usr/bin/env python
"""Generate the golden fixtures that pin the oracle to the TECS reference.

Runs oracle/_ref/ref_driver -- the reference's own headers compiled unmodified
against oracle/kokkos_shim (recipe: oracle/Makefile) -- on seeded inputs and
stores inputs and outputs as compressed .npz files next to this script:

  x0, p0          initial positions / polarities
  prm             cutoff, gabriel_c, min[3], max[3], k_rep, r_rep, k_adh, r_adh, k_pol, capacity, bin_scale
  pairs           directed (self, other) pairs of one full-step pass, in the reference's evaluation order
  dpos, dpol      per-cell deltas of that pass
  pos, pol        state after `steps` Simulation::take_step(dt) calls

Needs the reference sources (default /root/reference, override with
TECS_REFERENCE); run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from tecs_gb300 import workloads as wl  # noqa: E402

REF = Path(os.environ.get("TECS_REFERENCE", "/root/reference"))  # this script reads the reference where it lies
DRIVER = ROOT / "oracle" / "_ref" / "ref_driver"

# name: (driver scenario, oracle finder, symmetric, integrator, com, dims, polarity)
SCENARIOS = {
    "c1_small_euler": ("ba_euler_3", 1, 0, 0, 0, 3, 0),
    "bg_heun": ("bg_heun_3", 3, 0, 1, 0, 3, 0),
    "bg_heun_com": ("bg_heun_com_3", 3, 0, 1, 1, 3, 0),
    "bg_heun_clamped": ("bg_heun_3", 3, 0, 1, 0, 3, 0),
    "ba_heun_com": ("ba_heun_com_3", 1, 0, 1, 1, 3, 0),
    "bg_euler_com": ("bg_euler_com_3", 3, 0, 0, 1, 3, 0),
    "na_heun": ("na_heun_3", 0, 0, 1, 0, 3, 0),
    "ng_heun": ("ng_heun_3", 2, 0, 1, 0, 3, 0),
    "bgs_euler_com": ("bgs_euler_com_3", 3, 1, 0, 1, 3, 0),
    "bas_heun": ("bas_heun_3", 1, 1, 1, 0, 3, 0),
    "ngs_euler": ("ngs_euler_3", 2, 1, 0, 0, 3, 0),
    "nas_heun": ("nas_heun_3", 0, 1, 1, 0, 3, 0),
    "bg_heun_polarity": ("bg_heun_pol_3", 3, 0, 1, 0, 3, 1),
    "ng_euler_2d_points11": ("ng_euler_2", 2, 0, 0, 0, 2, 0),
    "bg_heun_2d": ("bg_heun_2", 3, 0, 1, 0, 2, 0),
    "nd_euler_2d": ("nd_euler_2", 4, 0, 0, 0, 2, 0),
    "nd_euler_2d_points11": ("nd_euler_2", 4, 0, 0, 0, 2, 0),
    "nd_heun_3d": ("nd_heun_3", 4, 0, 1, 0, 3, 0),
    "lk_bg_heun": ("lk_bg_heun_3", 3, 0, 1, 0, 3, 0),
    "lk_ba_euler_com": ("lk_ba_euler_com_3", 1, 0, 0, 1, 3, 0),
    # the reference's HDF5_Writer on a stepped run: its XDMF sidecar (lk_writer.xmf)
    "lk_writer": ("lk_writer_3", 3, 0, 1, 0, 3, 1),
    # the same without links: the grids' topology is then the cells as vertices
    "lk_writer_nolinks": ("lk_writer_3", 3, 0, 1, 0, 3, 1),
    # a GENERIC_FORCE law with the spring: final positions only
    "gen_bg_heun": ("gen_bg_heun_3", 3, 0, 1, 0, 3, 0),
    # a pairwise law that sets drag: final positions and old velocities
    "drag_bg_heun": ("drag_bg_heun_3", 3, 0, 1, 0, 3, 0),
    "drag_ba_euler_com": ("drag_ba_euler_com_3", 1, 0, 0, 1, 3, 0),
    # update functions between steps (run, run_links, init): positions, links, a DeviceVar count
    "upd_bg_heun": ("upd_bg_heun_3", 3, 0, 1, 0, 3, 0),
    # a config with a Scalar and a Vector field beyond the position: pos, u, w
    "fields_bg_heun": ("fields_bg_heun_3", 3, 0, 1, 0, 3, 0),
    "fields_ba_euler_com": ("fields_ba_euler_com_3", 1, 0, 0, 1, 3, 0),
}


def make_links(x, seed, n_links):
    """Protrusion-like links: cells joined to a random cell within 1.6, plus
    duplicates and self links (a == b, skipped by the reference)."""
    rng = np.random.default_rng(seed)
    from scipy.spatial import cKDTree

    t = cKDTree(x)
    out = []
    while len(out) < n_links:
        a = int(rng.integers(len(x)))
        near = [b for b in t.query_ball_point(x[a], 1.6) if b != a]
        if near:
            out.append((a, int(rng.choice(near))))
    out += [out[0], out[1], (5, 5), (len(x) - 1, len(x) - 1)]
    return np.array(out, np.uint32)


def main_cpp_points():
    """The 11-point 2-D table of the reference's main.cpp (its Gabriel demo fixture)."""
    text = (REF / "main.cpp").read_text()
    block = text[text.index("pos[n_cells][2]"):]
    block = block[: block.index("};")]
    pts = re.findall(r"\{\s*(-?\d+\.\d+),\s*(-?\d+\.\d+)\s*\}", block)
    return np.array(pts, dtype=np.float32)


def inputs(name):
    """(x0, p0, prm, steps, dt) for one scenario."""
    prm = np.zeros(16, np.float32)
    prm[0], prm[1] = 1.0, 0.8
    prm[8:13] = (2.0, 0.7, 0.5, 0.8, 0.0)
    prm[14] = 1.0
    p0 = None
    if name == "c1_small_euler":
        x = wl.ball(1000, 0, radius=5.0)
        mn, mx, steps, dt = (-6,) * 3, (6,) * 3, 1000, 0.1
    elif name in ("bg_heun", "bg_heun_com"):
        x = wl.ball(3000, 1)
        mn, mx = wl.bounds_for(x)
        steps, dt = 20, 0.05
        if name == "bg_heun_com":
            prm[13] = 3150
    elif name == "bg_heun_clamped":
        # the default +-20 grid around a ball of radius 26: outside cells land in edge bins
        x = wl.ball(2000, 12, radius=26.0)
        mn, mx, steps, dt = (-20,) * 3, (20,) * 3, 5, 0.05
    elif name in ("ba_heun_com", "bg_euler_com", "bgs_euler_com", "bas_heun"):
        seed = {"ba_heun_com": 3, "bg_euler_com": 4, "bgs_euler_com": 7, "bas_heun": 8}[name]
        x = wl.ball(2000, seed)
        mn, mx = wl.bounds_for(x)
        steps, dt = (10, 0.05) if name in ("ba_heun_com", "bg_euler_com") else (5, 0.05)
        if name in ("ba_heun_com", "bgs_euler_com"):
            prm[13] = 2100
    elif name == "na_heun":
        x = wl.ball(600, 5)
        mn, mx, steps, dt = (-20,) * 3, (20,) * 3, 5, 0.05
    elif name == "nas_heun":
        x = wl.ball(500, 20)
        mn, mx, steps, dt = (-20,) * 3, (20,) * 3, 4, 0.05
    elif name in ("ng_heun", "ngs_euler"):
        x = wl.ball(400 if name == "ng_heun" else 300, 6 if name == "ng_heun" else 9)
        mn, mx, steps, dt = (-20,) * 3, (20,) * 3, 3, 0.05
    elif name == "bg_heun_polarity":
        x = wl.sheet(2000, 10)
        p0 = wl.outward_polarity(x, 10)
        mn, mx = wl.bounds_for(x)
        prm[12] = 0.2
        steps, dt = 5, 0.05
    elif name in ("ng_euler_2d_points11", "nd_euler_2d_points11"):
        x = main_cpp_points()
        prm[0] = 2.5
        mn, mx, steps, dt = (-20, -20, 0), (20, 20, 0), 3, 0.01
    elif name == "bg_heun_2d":
        x = np.ascontiguousarray(wl.ball(1500, 13)[:, :2] * 0.4)
        m = float(np.ceil(np.abs(x).max() + 2))
        mn, mx, steps, dt = (-m, -m, 0), (m, m, 0), 10, 0.05
    elif name == "nd_euler_2d":
        x = np.ascontiguousarray(wl.ball(120, 14)[:, :2])
        mn, mx, steps, dt = (-20, -20, 0), (20, 20, 0), 4, 0.02
    elif name in ("lk_bg_heun", "lk_ba_euler_com"):
        x = wl.ball(2000, 16)
        mn, mx = wl.bounds_for(x)
        prm[15] = 0.2  # link strength
        steps, dt = (10, 0.05) if name == "lk_bg_heun" else (20, 0.05)
        if name == "lk_ba_euler_com":
            prm[13] = 2100
    elif name in ("lk_writer", "lk_writer_nolinks"):
        x = wl.sheet(60 if name == "lk_writer" else 45, 18)
        p0 = wl.outward_polarity(x, 18)
        mn, mx = wl.bounds_for(x)
        steps, dt = 2, 0.05
    elif name == "nd_heun_3d":
        x = wl.ball(48, 15)
        mn, mx, steps, dt = (-20,) * 3, (20,) * 3, 3, 0.05
    elif name == "gen_bg_heun":
        x = wl.ball(2000, 19)
        mn, mx = wl.bounds_for(x)
        steps, dt = 10, 0.05
    elif name in ("fields_bg_heun", "fields_ba_euler_com"):
        x = wl.ball(1500, 24 if name == "fields_bg_heun" else 25)
        mn, mx = wl.bounds_for(x)
        steps, dt = 10, 0.05
        if name == "fields_ba_euler_com":
            prm[13] = 1600
    elif name == "upd_bg_heun":
        x = wl.ball(800, 23)
        mn, mx = wl.bounds_for(x)
        steps, dt = 3, 0.05
    elif name in ("drag_bg_heun", "drag_ba_euler_com"):
        x = wl.ball(1500, 21 if name == "drag_bg_heun" else 22)
        mn, mx = wl.bounds_for(x)
        steps, dt = 8, 0.05
        if name == "drag_ba_euler_com":
            prm[13] = 1600
    else:
        raise KeyError(name)
    prm[2:5] = mn
    prm[5:8] = mx
    return np.ascontiguousarray(x, np.float32), p0, prm, steps, dt


# grid-query fixtures: the reference's acceleration::Grid queried at seeded
# points; name: (driver scenario, dims, points, queries, bin size, search radius, half-width of the bounds)
GRID = {
    "grid_q_3d": ("grid_3", 3, 3000, 600, 0.75, 1.3, 7.0),
    "grid_q_2d": ("grid_2", 2, 1500, 400, 1.0, 1.6, 12.0),
}


def grid_inputs(name):
    scen, dims, n, m, bin_size, radius, half = GRID[name]
    rng = np.random.default_rng(40 + dims)
    # points in a ball slightly larger than the bounds (the outside ones are
    # clamped into edge bins), queries over a wider box (some far from every point)
    x = (wl.ball(n, 41 + dims)[:, :dims] * (half * 1.15 / wl.ball_radius(n))).astype(np.float32)
    q = rng.uniform(-half * 1.3, half * 1.3, (m, dims)).astype(np.float32)
    q[: m // 4] = x[rng.integers(0, n, m // 4)]  # some queries exactly at points
    draws = rng.integers(0, 2 ** 32, m, dtype=np.uint64).astype(np.uint32)
    prm = np.zeros(16, np.float32)
    prm[0], prm[1] = bin_size, radius
    prm[2:2 + dims] = -half
    prm[5:5 + dims] = half
    return np.ascontiguousarray(x), np.ascontiguousarray(q), draws, prm


def run_grid(name):
    scen, dims = GRID[name][0], GRID[name][1]
    x, q, draws, prm = grid_inputs(name)
    with tempfile.TemporaryDirectory() as td:
        inp = Path(td) / "in.bin"
        with open(inp, "wb") as f:
            np.array([len(x), dims, 0], np.uint32).tofile(f)
            prm.tofile(f)
            x.tofile(f)
            np.array([len(q)], np.uint32).tofile(f)
            q.tofile(f)
            draws.tofile(f)
        out = Path(td) / "out"
        subprocess.run([str(DRIVER), scen, str(inp), str(out), "0", "0"], check=True)
        res = {"x": x, "q": q, "draws": draws, "prm": prm}
        for k in ("near1", "near2", "rbins", "rrad", "rfilt"):
            res[k] = np.fromfile(f"{out}.{k}", np.int32)
    np.savez_compressed(HERE / f"{name}.npz", **res)
    return res


# whole reference programs (examples/<program>.cpp, unmodified) run on the
# shim with their datasets dumped: name -> (program, snapshots kept, stop after K groups or None)
EXAMPLES = {
    "ex_springs": ("springs", "first_last", None),
    "ex_epithelium": ("epithelium", "first_last", None),
    "ex_polarization": ("polarization", "first_last", None),
    "ex_growth_w_wall": ("growth_w_wall", "first_last", None),
    "ex_delaunay_spheroid": ("delaunay_spheroid", "first", 1),
}


def run_example(name):
    prog, keep, stop = EXAMPLES[name]
    exe = ROOT / "oracle" / "_ref" / "examples" / prog
    with tempfile.TemporaryDirectory() as td:
        (Path(td) / "output").mkdir()
        dump = Path(td) / "dump"
        dump.mkdir()
        env = dict(os.environ, TECS_SHIM_DUMP=str(dump))
        if stop:
            env["TECS_SHIM_STOP_AFTER"] = str(stop)
        subprocess.run([str(exe)], cwd=td, env=env, check=True, stdout=subprocess.DEVNULL)
        groups = sorted({f.name.split(".")[0] for f in dump.iterdir()}, key=lambda g: int(g[1:]))
        res = {"counts": np.array([(dump / f"{g}.position.bin").stat().st_size // 12 for g in groups], np.int64)}
        for g in ([groups[0], groups[-1]] if keep == "first_last" else [groups[0]]):
            for field, dtype, cols in (("position", np.float32, 3), ("polarity", np.float32, 2),
                                       ("links", np.uint32, 2)):
                f = dump / f"{g}.{field}.bin"
                if f.exists():
                    res[f"{g}_{field}"] = np.fromfile(f, dtype).reshape(-1, cols)
        res["groups"] = np.array([int(g[1:]) for g in groups], np.int64)
    np.savez_compressed(HERE / f"{name}.npz", **res)
    return res


# the reference's predefined force functions (forces/predefined.hpp) at a
# table of distances: name -> driver scenario
LAWS = {"laws_predefined": "laws"}


def run_laws(name):
    """Distances 0..2.5 (every branch point of the seven laws, the points
    beside them, and a random spread) with displacements of those lengths."""
    rng = np.random.default_rng(11)
    marks = np.array([0.0, 0.6, 0.8, 0.9, 1.0, 1.1, 1.3, 1.4, 1.6, 1.8, 2.0], np.float32)
    d = np.concatenate([marks, np.nextafter(marks, np.float32(-1)), np.nextafter(marks, np.float32(3)),
                        rng.uniform(0.0, 2.5, 200).astype(np.float32)]).astype(np.float32)
    d = np.abs(d)
    u = rng.normal(size=(len(d), 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    disp = (u * d[:, None]).astype(np.float32)
    with tempfile.TemporaryDirectory() as td:
        inp = Path(td) / "in.bin"
        with open(inp, "wb") as f:
            np.array([len(d)], np.uint32).tofile(f)
            d.tofile(f)
            disp.tofile(f)
        out = Path(td) / "out"
        subprocess.run([str(DRIVER), LAWS[name], str(inp), str(out), "0", "0"], check=True)
        res = np.fromfile(f"{out}.laws", np.float32).reshape(len(d), 28)
    r = {"d": d, "disp": disp, "magnitude": res[:, :7], "vector": res[:, 7:].reshape(len(d), 7, 3)}
    np.savez_compressed(HERE / f"{name}.npz", **r)
    return r


def run(name):
    if name in LAWS:
        return run_laws(name)
    if name in GRID:
        return run_grid(name)
    if name in EXAMPLES:
        return run_example(name)
    scen, *_rest, dims, pol = SCENARIOS[name]
    x, p0, prm, steps, dt = inputs(name)
    if name == "lk_writer_nolinks":
        links = np.zeros((0, 2), np.uint32)
    elif scen.startswith("lk_"):
        links = make_links(x, 17, 30 if name == "lk_writer" else 400)
    else:
        links = None
    with tempfile.TemporaryDirectory() as td:
        inp = Path(td) / "in.bin"
        with open(inp, "wb") as f:
            np.array([len(x), dims, 1 if p0 is not None else 0], np.uint32).tofile(f)
            prm.tofile(f)
            x.tofile(f)
            if p0 is not None:
                p0.astype(np.float32).tofile(f)
            if links is not None:
                np.array([len(links)], np.uint32).tofile(f)
                links.tofile(f)
        out = Path(td) / "out"
        subprocess.run([str(DRIVER), scen, str(inp), str(out), str(steps), repr(dt)], check=True)
        if scen == "lk_writer_3":
            (HERE / f"{name}.xmf").write_bytes(Path(f"{out}.xmf").read_bytes())
            res = {"x0": x, "p0": p0, "prm": prm, "steps": np.int64(steps), "dt": np.float64(dt), "links": links}
            np.savez_compressed(HERE / f"{name}.npz", **res)
            return res
        res = {"x0": x, "prm": prm, "steps": np.int64(steps), "dt": np.float64(dt),
               "pos": np.fromfile(f"{out}.pos", np.float32).reshape(-1, dims)}
        if links is not None:
            res["links"] = links
        elif scen.startswith("gen_"):
            pass
        elif scen.startswith("drag_"):
            res["ov"] = np.fromfile(f"{out}.ov", np.float32).reshape(-1, dims)
        elif scen.startswith("fields_"):
            res["u"] = np.fromfile(f"{out}.u", np.float32)
            res["w"] = np.fromfile(f"{out}.w", np.float32).reshape(-1, dims)
        elif scen.startswith("upd_"):
            res["links"] = np.fromfile(f"{out}.links", np.uint32).reshape(-1, 2)
            res["hits"] = np.fromfile(f"{out}.hits", np.int32)
        else:
            res["pairs"] = np.fromfile(f"{out}.pairs", np.uint32).reshape(-1, 2)
            res["dpos"] = np.fromfile(f"{out}.dpos", np.float32).reshape(-1, dims)
        if p0 is not None:
            res["p0"] = p0
            res["dpol"] = np.fromfile(f"{out}.dpol", np.float32).reshape(-1, 2)
            res["pol"] = np.fromfile(f"{out}.pol", np.float32).reshape(-1, 2)
    np.savez_compressed(HERE / f"{name}.npz", **res)
    return res


def main():
    if not REF.exists():
        sys.exit(f"reference sources not found at {REF}")
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), f"REF={REF}", "all", "examples"], check=True)
    names = sys.argv[1:] or list(SCENARIOS) + list(GRID) + list(EXAMPLES) + list(LAWS)
    manifest = {}
    for name in names:
        r = run(name)
        if name in LAWS:
            manifest[name] = {"scenario": LAWS[name], "distances": int(len(r["d"]))}
            print(name, manifest[name])
            continue
        if name in GRID:
            manifest[name] = {"scenario": GRID[name][0], "points": int(len(r["x"])), "queries": int(len(r["q"]))}
            print(name, manifest[name])
            continue
        if name in EXAMPLES:
            manifest[name] = {"program": EXAMPLES[name][0], "snapshots": int(len(r["groups"])),
                              "agents_last": int(r["counts"][-1])}
            print(name, manifest[name])
            continue
        manifest[name] = {"scenario": SCENARIOS[name][0], "cells": int(len(r["x0"])),
                          "pairs": int(len(r["pairs"])) if "pairs" in r else None,
                          "links": int(len(r["links"])) if "links" in r else None,
                          "steps": int(r["steps"]), "dt": float(r["dt"])}
        print(name, manifest[name])
    old = {}
    mf = HERE / "manifest.json"
    if mf.exists():
        old = json.loads(mf.read_text())
    old.update(manifest)
    mf.write_text(json.dumps(old, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
