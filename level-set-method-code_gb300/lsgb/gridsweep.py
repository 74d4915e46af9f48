"""Stage-kernel throughput of the FP32 3D handle against the grid size.

One solver per cubic grid n^3 on the configuration-3 fields (perturbed
sphere, curl of a random vector potential, S_L = 0.2, CFL 0.5), its tile
shape picked by lsgb_solver_autotune, then the average stage launch over
20 RK3 steps with CUDA events on the solver's stream.  The grid sizes pair
neighbours that differ in what the stage kernel can do with them:

  * nx % 4 == 0: rows are 16-byte aligned and the planes are staged by
    bulk-tensor copies; otherwise by cp.async element copies;
  * n just above a multiple of the 32 x 16 tile: the last tile row and
    column are nearly empty;
  * small grids: one launch has too few tiles to fill 152 SMs, and its
    duration approaches the launch latency.

    python level-set-method-code_gb300/lsgb/gridsweep.py --json sizes.json
"""
from __future__ import annotations

import argparse
import json
import os
import sys

if __package__ in (None, ""):
    _pkg = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, _pkg)
    sys.path.insert(0, os.path.dirname(_pkg))

import lsgb  # noqa: E402
from lsgb import synthetic as syn  # noqa: E402

SIZES = (192, 188, 187, 152, 151, 130, 128, 65, 64, 41, 40)


def sweep(sizes=SIZES, steps: int = 20) -> dict:
    out = {}
    for n in sizes:
        wl = syn.config3(n)
        p = lsgb.params(3, n, n, n, s_l=wl.s_l, enable_reinit=True, reinit_interval=5, reinit_iterations=2)
        with lsgb.Solver(p, "f32") as s:
            s.synth(syn.to_device_desc(wl))
            s.compute_dt(0.5)
            tile, _ = s.autotune(3)
            s.advance(5)
            s.enable_timing(True)
            s.advance(steps)
            st, sn, _, _ = s.kernel_times()
            s.enable_timing(False)
        ms = st / sn
        out[str(n)] = {"stage_ms": ms, "gcell_stage_per_s": n ** 3 / (ms * 1e-3) / 1e9, "tile": tile,
                       "bulk_tensor": n % 4 == 0}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default=",".join(str(n) for n in SIZES))
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    r = sweep([int(x) for x in a.sizes.split(",")], a.steps)
    for n, v in r.items():
        print(f"{n:>5}^3  {v['stage_ms']:.4f} ms/stage  {v['gcell_stage_per_s']:6.1f} Gcell/s  tile {v['tile']}"
              f"  {'bulk-tensor' if v['bulk_tensor'] else 'cp.async'}")
    if a.json:
        with open(a.json, "w") as f:
            json.dump(r, f, indent=1)


if __name__ == "__main__":
    main()
