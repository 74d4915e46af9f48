"""Precision report of the FP32-bulk form against the plain FP64 form.

Runs the same seeded workload (configuration 3: perturbed sphere, curl of a
random vector potential, S_L = 0.2, CFL 0.5, HCR-2 every 5 steps with 2
pseudo-steps) in both precisions from identical initial fields and compares
the two G fields at checkpoints:

  * L_inf and L2 of G32 - G64 over the cells within 3 cells of the front
    (|G64| < 3 dx), and L_inf over all cells;
  * the zero-level-set position error: on every grid edge (x, y and z) where
    both fields change sign, the linear-interpolated crossing point
    t = G_a / (G_a - G_b) of each run, reported as max and mean |t32 - t64|
    in units of dx;
  * the enclosed volume (cells with G < 0, times the cell volume) and its
    smoothed-Heaviside variant sum 1/2 (1 - tanh(G / (1.5 dx))) dV, both runs,
    and their drift from the initial field.

    python level-set-method-code_gb300/lsgb/precision.py --n 512 --steps 1000 --every 200 --json out.json
    python level-set-method-code_gb300/lsgb/precision.py --config 2 --n 256 --steps 500 --every 100 --json c2.json
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

if __package__ in (None, ""):
    _pkg = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, _pkg)
    sys.path.insert(0, os.path.dirname(_pkg))

import lsgb  # noqa: E402
from lsgb import synthetic as syn  # noqa: E402


def _grad_mag(g: np.ndarray, dx: float) -> np.ndarray:
    s = 0.0
    for ax in range(g.ndim):
        s = s + ((np.roll(g, -1, ax) - np.roll(g, 1, ax)) / (2 * dx)) ** 2
    return np.sqrt(s)


def crossing_error(g32: np.ndarray, g64: np.ndarray, dx: float = 1.0):
    """Over the grid edges crossed in both fields, all axes: max / mean of
    |t32 - t64| (the along-edge shift of the linear-interpolated crossing, in
    dx), and max / mean of the normal displacement of the front,
    |t32 - t64| |G64_a - G64_b| / (dx |grad G64|) (in dx).  The along-edge
    shift is large on edges the front grazes (|G_a - G_b| << dx |grad G|);
    the normal displacement is the geometric position error."""
    worst, total, count = 0.0, 0.0, 0
    nworst, ntotal = 0.0, 0.0
    gm = _grad_mag(g64, dx)
    for ax in range(g64.ndim):
        a64, b64 = g64, np.roll(g64, -1, axis=ax)
        a32, b32 = g32, np.roll(g32, -1, axis=ax)
        both = (a64 * b64 < 0) & (a32 * b32 < 0)
        if not both.any():
            continue
        t64 = a64[both] / (a64[both] - b64[both])
        t32 = a32[both] / (a32[both] - b32[both])
        e = np.abs(t32 - t64)
        ge = 0.5 * (gm[both] + np.roll(gm, -1, axis=ax)[both])
        en = e * np.abs(a64[both] - b64[both]) / (dx * np.maximum(ge, 1e-300))
        worst = max(worst, float(e.max()))
        total += float(e.sum())
        nworst = max(nworst, float(en.max()))
        ntotal += float(en.sum())
        count += e.size
    mean = total / count if count else 0.0
    nmean = ntotal / count if count else 0.0
    return worst, mean, count, nworst, nmean


def volumes(g: np.ndarray, dx: float):
    dv = dx ** g.ndim
    sharp = float(np.count_nonzero(g < 0)) * dv
    eps = 1.5 * dx
    smooth = float(np.sum(0.5 * (1.0 - np.tanh(g / eps)))) * dv
    return sharp, smooth


def compare(g32: np.ndarray, g64: np.ndarray, dx: float) -> dict:
    d = np.abs(g32 - g64)
    band = np.abs(g64) < 3 * dx
    cmax, cmean, cn, nmax, nmean = crossing_error(g32, g64, dx)
    v64, s64 = volumes(g64, dx)
    v32, s32 = volumes(g32, dx)
    return {
        "linf_G": float(d.max()),
        "linf_G_band3": float(d[band].max()) if band.any() else None,
        "l2_G_band3": float(np.sqrt(np.mean(d[band] ** 2))) if band.any() else None,
        "linf_G_band3_over_dx": float(d[band].max() / dx) if band.any() else None,
        "front_position_err_max_dx": cmax,
        "front_position_err_mean_dx": cmean,
        "front_normal_err_max_dx": nmax,
        "front_normal_err_mean_dx": nmean,
        "front_edges_compared": cn,
        "volume_f64": v64, "volume_f32": v32,
        "volume_smooth_f64": s64, "volume_smooth_f32": s32,
    }


def run(n: int = 512, steps: int = 1000, every: int = 200, cfl: float = 0.5, config: int = 3,
        n_modes: int = 24) -> dict:
    wl = syn.sphere_config(config, n, n_modes, 0.2)
    p = lsgb.params(3, n, n, n, s_l=wl.s_l, enable_reinit=True, reinit_interval=5, reinit_iterations=2)
    s64 = lsgb.Solver(p, "f64")
    s32 = lsgb.Solver(p, "f32")
    desc = syn.to_device_desc(wl)
    s64.synth(desc)
    s32.synth(desc)
    dt = s64.compute_dt(cfl)
    s32.set_dt(dt)
    dx = 1.0 / n
    g0 = s64.get_G(layout="compact")
    v0, vs0 = volumes(g0, dx)
    del g0
    report = {"config": config, "n": n, "steps": steps, "dt": dt, "cfl": cfl, "volume_initial": v0,
              "volume_smooth_initial": vs0, "checkpoints": []}
    done = 0
    t64 = t32 = 0.0
    while done < steps:
        seg = min(every, steps - done)
        a = time.perf_counter()
        s64.advance(seg)
        s64.volume()  # synchronises
        t64 += time.perf_counter() - a
        a = time.perf_counter()
        s32.advance(seg)
        s32.volume()
        t32 += time.perf_counter() - a
        done += seg
        g64 = s64.get_G(layout="compact")
        g32 = s32.get_G(layout="compact")
        c = compare(g32, g64, dx)
        c["step"] = done
        c["volume_drift_f64"] = (c["volume_f64"] - v0) / v0
        c["volume_drift_f32"] = (c["volume_f32"] - v0) / v0
        report["checkpoints"].append(c)
        print(json.dumps(c), flush=True)
        del g64, g32
    report["seconds_f64"] = t64
    report["seconds_f32"] = t32
    s64.close()
    s32.close()
    return report


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--every", type=int, default=200)
    ap.add_argument("--config", type=int, default=3, help="seed family: 3 (24 modes) or 2 (16 modes)")
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    import __graft_entry__
    __graft_entry__.build_library()
    r = run(a.n, a.steps, a.every, config=a.config, n_modes=24 if a.config == 3 else 16)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(r, f, indent=2)
    print(json.dumps({k: v for k, v in r.items() if k != "checkpoints"}))


if __name__ == "__main__":
    main()
