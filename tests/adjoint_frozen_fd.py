"""Finite differences of the adjoint workload's forward map with its
switching decisions frozen at the base run (CPU, the oracle port), against
the FP64 discrete adjoint's directional derivatives <dL/dS_L, d>.

The discrete adjoint differentiates the forward with its piecewise choices
held at the base run: the upwind branch u_eff >= 0 per axis, the Godunov
one-sided choice of the HCR-2 pseudo-step, the crossing flags and the
stability mask.  A central difference of the free forward map steps across
those switching sets and picks up jumps no derivative contains.  Here the
oracle port records the base run's decisions (its decision tape) and replays
them in the perturbed runs, so the map being differenced is the one the
adjoint differentiates.  The port's base run is bit-identical to the GPU
FP64 forward, so both see the same decisions.

Workload: the adjoint workload (lsgb.adjoint.workload: 192^3, 300 steps,
HCR-2 every 10 x 2, S_L(x) = 0.15 + 0.05 f(x)); loss
L = 1/2 sum (H(G_T) - H(G_target))^2 dV, H(g) = (1 - tanh(g / 1.5 dx)) / 2.

    python tests/adjoint_frozen_fd.py --adjoint tests/golden/adjoint_directional_192.json \
        --dirs 32 --rel-step 1e-4 --json fd.json

About 1.6 minutes of 8 host cores per forward run at 192^3; tape memory
about 7 GB.  Results are written after every direction.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for _p in (ROOT, os.path.join(ROOT, "level-set-method-code_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

from oracle import Oracle, Problem  # noqa: E402


def ghost(a):
    return np.ascontiguousarray(np.pad(a, 3, mode="wrap"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--adjoint", required=True, help="JSON of lsgb/adjoint.py --directional")
    ap.add_argument("--dirs", type=int, default=32)
    ap.add_argument("--rel-step", type=float, nargs="+", default=[1e-4])
    ap.add_argument("--extra", default="", help="more (dir:rel_step) pairs, comma separated")
    ap.add_argument("--json", required=True)
    a = ap.parse_args()
    from lsgb import adjoint as adj
    ref = json.load(open(a.adjoint))
    n, steps = ref["n"], ref["steps"]
    p, G0, u, v, w, sl, sl_t = adj.workload(n, steps)
    pb = Problem(nx=n, ny=n, nz=n, dim=3, dx=p.dx, dy=p.dy, dz=p.dz, dt=p.dt, s_l=p.s_l, epsilon=p.epsilon,
                 enable_reinit=True, reinit_interval=p.reinit_interval, reinit_iterations=p.reinit_iterations,
                 reinit_dtau=p.reinit_dtau, reinit_beta=p.reinit_beta)
    orc = Oracle("port")
    G0g = ghost(G0)
    u, v, w = (orc.apply_bc(pb, ghost(x)) for x in (u, v, w))
    eps, dv = 1.5 * p.dx, p.dx * p.dy * p.dz
    inner = (slice(3, -3),) * 3
    H = lambda g: 0.5 * (1.0 - np.tanh(g / eps))

    def forward(slg):
        G = G0g.copy()
        orc.run_filled(pb, steps, G, u, v, w, sl=slg)
        return G[inner]

    t0 = time.time()
    Ht = H(forward(ghost(sl_t)))
    loss = lambda GT: 0.5 * float(np.sum((H(GT) - Ht) ** 2)) * dv
    cells = n ** 3
    n_re = (steps - 1) // p.reinit_interval
    stage = np.zeros((3 * steps, cells), np.uint8)
    pseudo = np.zeros((p.reinit_iterations * n_re, cells), np.uint8)
    flags = np.zeros((n_re, cells), np.uint8)
    orc.tape("record", stage, pseudo, flags)
    L0 = loss(forward(ghost(sl)))
    counts = orc.tape_counts()
    orc.tape("off")
    assert counts == (3 * steps, p.reinit_iterations * n_re, n_re, 0), counts
    out = {"n": n, "steps": steps, "loss_port": L0, "loss_gpu": ref["loss_f64"],
           "seconds_setup": time.time() - t0, "rows": []}
    pairs = [(q, rs) for rs in a.rel_step for q in range(a.dirs)]
    for item in filter(None, a.extra.split(",")):
        q, rs = item.split(":")
        pairs.append((int(q), float(rs)))
    norm_sl = float(np.linalg.norm(sl))
    for q, rs in pairs:
        d = adj.direction(sl.shape[::-1], q, ref["seed"])
        h = rs * norm_sl
        L = []
        for sgn in (1.0, -1.0):
            orc.tape("replay", stage, pseudo, flags)
            L.append(loss(forward(ghost(sl + sgn * h * d))))
            orc.tape("off")
        fd = (L[0] - L[1]) / (2 * h)
        ad = ref["adjoint"][q]
        out["rows"].append({"dir": q, "rel_step": rs, "fd": fd, "adjoint": ad,
                            "rel_err": abs(fd - ad) / max(abs(fd), 1e-300)})
        errs = [r["rel_err"] for r in out["rows"] if r["rel_step"] == rs]
        out[f"rel_err_median@{rs:g}"] = float(np.median(errs))
        out[f"rel_err_max@{rs:g}"] = float(np.max(errs))
        out["seconds"] = time.time() - t0
        with open(a.json, "w") as f:
            json.dump(out, f, indent=1)
        print(json.dumps(out["rows"][-1]), flush=True)


if __name__ == "__main__":
    main()
