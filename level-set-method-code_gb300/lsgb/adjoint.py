"""Gradients through the level-set solver: a torch autograd Function over the
discrete adjoint of the C ABI (lsgb_adjoint_*), the adjoint workload
(192^3 perturbed sphere, spatially varying flame speed), and the gradient
check against central finite differences.

Adjoint workload (seeded, synthetic):
  * G0 and u as the 3D benchmark sphere (8 harmonic perturbations, curl of a
    16-mode random vector potential scaled to max|u| = 1);
  * S_L(x) = 0.15 + 0.05 f(x), f an 8-mode random Fourier field with
    max|f| = 1 over the grid; the target front comes from a forward run with
    another seed of f;
  * L = 1/2 sum (H(G_T) - H(G_target))^2 dV, H(g) = (1 - tanh(g / eps)) / 2,
    eps = 1.5 dx; 300 steps, CFL 0.5, HCR-2 every 10 steps, checkpoints every 20.

    python level-set-method-code_gb300/lsgb/adjoint.py --n 192 --steps 300 --dirs 32 --json out.json
"""
from __future__ import annotations

import argparse
import json
import math
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

CONFIG = 5


def fourier_field(n, seed: int, n_modes: int = 8, kmax: int = 4) -> np.ndarray:
    """Random Fourier field sum_m a_m cos(2 pi k_m . x + phi_m) on the cell
    centres x_i = i / n (compact layout, shape (nz, ny, nx) or (ny, nx)),
    normalised to max |f| = 1."""
    n = tuple(n)
    dim = len(n)
    rng = np.random.default_rng(seed)
    axes = [np.arange(q, dtype=np.float64) / q for q in n]
    grids = np.meshgrid(*axes[::-1], indexing="ij")[::-1]  # x, y(, z) in (.., ny, nx) order
    f = np.zeros(n[::-1], dtype=np.float64)
    m = 0
    while m < n_modes:
        k = rng.integers(-kmax, kmax + 1, size=dim)
        if not 0 < int(np.sum(k * k)) <= kmax * kmax:
            continue
        a = rng.standard_normal()
        ph = rng.uniform(0.0, 2.0 * math.pi)
        arg = sum(2.0 * math.pi * float(k[q]) * grids[q] for q in range(dim))
        f += a * np.cos(arg + ph)
        m += 1
    return f / np.abs(f).max()


def sl_field(n, seed: int) -> np.ndarray:
    return 0.15 + 0.05 * fourier_field(n, seed)


def workload(n: int = 192, steps: int = 300, dim: int = 3, cfl: float = 0.5, reinit_interval: int = 10,
             reinit_iterations: int = 2, reinit: bool = True, bc=None):
    """(params, G0, u, v, w, sl, sl_target) of the adjoint workload; fields in
    the compact layout, FP64 host arrays.  bc: boundary per axis ("periodic"
    or "zero_gradient", x first; default periodic everywhere)."""
    if dim == 3:
        wl = syn.sphere_config(CONFIG, n, 16, 0.15)
    else:
        rng = np.random.default_rng(syn.seed_for(CONFIG, 1))
        wl = syn.Workload(dim=2, n=(n, n), s_l=0.15, center=(0.5, 0.5, 0.0), r0=0.25)
        wl.vel_k, wl.vel_c, wl.vel_phase = syn.draw_modes(rng, 2, 8)
    G, u, v, w = syn.host_fields(wl)
    inner = (slice(3, -3),) * dim
    G, u, v = G[inner].copy(), u[inner].copy(), v[inner].copy()
    w = w[inner].copy() if dim == 3 else None
    grid = (n,) * dim
    sl = sl_field(grid, syn.seed_for(CONFIG, 100))
    sl_t = sl_field(grid, syn.seed_for(CONFIG, 200))
    speed = np.abs(u) + np.abs(v) + (np.abs(w) if dim == 3 else 0.0)
    dt = cfl * (1.0 / n) / (float(speed.max()) + float(max(sl.max(), sl_t.max())))
    bcs = {"bc_" + a: b for a, b in zip("xyz", bc or ())}
    p = lsgb.params(dim, n, n, n if dim == 3 else 1, dx=1.0 / n, dy=1.0 / n, dz=1.0 / n, s_l=0.15, dt=dt,
                    enable_reinit=reinit, reinit_interval=reinit_interval, reinit_iterations=reinit_iterations,
                    **bcs)
    return p, G, u, v, w, sl, sl_t


class Problem:
    """Solver + adjoint over fixed G0 and velocity; loss(sl) and grad(sl)."""

    def __init__(self, p, G0, u, v, w, precision: str = "f64", checkpoint: int = 20):
        self.p, self.G0, self.u, self.v, self.w = p, G0, u, v, w
        self.eps = 1.5 * p.dx
        self.s = lsgb.Solver(p, precision)
        self.a = lsgb.Adjoint(self.s, checkpoint)

    def close(self):
        self.a.close()
        self.s.close()

    def run(self, sl, n_steps: int, record: bool = False):
        self.s.set_fields(self.G0, self.u, self.v, self.w, layout="compact")
        self.s.set_sl_field(sl, layout="compact")
        self.s.step = 0
        if record:
            self.a.forward(n_steps)
        else:
            self.s.advance(n_steps)

    def target(self, sl_t, n_steps: int):
        self.run(sl_t, n_steps)
        gt = self.s.get_G(layout="compact")
        self.a.set_target(gt, self.eps, layout="compact")
        return gt

    def loss(self, sl, n_steps: int) -> float:
        self.run(sl, n_steps)
        return self.a.loss()

    def gradient(self, sl, n_steps: int):
        self.run(sl, n_steps, record=True)
        L = self.a.loss(seed=True)
        self.a.backward()
        return L, self.a.grad("sl")


def fd_check(prob: Problem, sl, n_steps: int, n_dirs: int, rel_step=1e-3, seed: int = 7):
    """Central differences of L along n_dirs random smooth unit directions d
    (||d||_2 = 1 over the cells), step h = rel_step * ||S_L||_2 (one step or a
    list of steps), against <dL/dS_L, d> of the adjoint."""
    L, g = prob.gradient(sl, n_steps)
    steps = [rel_step] if np.isscalar(rel_step) else list(rel_step)
    rows = []
    for q in range(n_dirs):
        d = direction(sl.shape[::-1], q, seed)
        ad = float(np.sum(g * d))
        for rs in steps:
            h = rs * float(np.linalg.norm(sl))
            lp = prob.loss(sl + h * d, n_steps)
            lm = prob.loss(sl - h * d, n_steps)
            fd = (lp - lm) / (2 * h)
            rows.append({"dir": q, "rel_step": rs, "fd": fd, "adjoint": ad,
                         "rel_err": abs(fd - ad) / max(abs(fd), 1e-300)})
    return L, g, rows


def direction(shape_xyz, q: int, seed: int = 7) -> np.ndarray:
    """The q-th smooth random unit direction of the finite-difference checks
    (an 8-mode Fourier field, ||d||_2 = 1 over the cells)."""
    d = fourier_field(shape_xyz, seed * 1000 + q)
    return d / np.linalg.norm(d)


def directional(n: int = 192, steps: int = 300, dirs: int = 32, checkpoint: int = 20, seed: int = 7) -> dict:
    """<dL/dS_L, d_q> of the FP64 adjoint on the adjoint workload for the
    directions d_0 .. d_{dirs-1}, with the loss.  The discrete adjoint holds
    the forward's switching decisions fixed at the base run (the upwind
    branches, the Godunov choices, the crossing flags and the stability
    mask), so these are derivatives of the forward map with those decisions
    frozen."""
    p, G0, u, v, w, sl, sl_t = workload(n, steps)
    prob = Problem(p, G0, u, v, w, "f64", checkpoint)
    prob.a.set_grads(sl=True, velocity=False)
    prob.target(sl_t, steps)
    L, g = prob.gradient(sl, steps)
    prob.close()
    ad = [float(np.sum(g * direction(sl.shape[::-1], q, seed))) for q in range(dirs)]
    return {"n": n, "steps": steps, "checkpoint": checkpoint, "dt": p.dt, "seed": seed, "loss_f64": L,
            "adjoint": ad, "grad_l2": float(np.linalg.norm(g))}


# -- torch ------------------------------------------------------------------
def rollout(G0, sl, u, v, w, p, n_steps: int, precision: str = "f64", checkpoint: int = 20):
    """G_T = n_steps solver steps from G0 with flame-speed field sl and
    velocity (u, v, w); all torch float64 CUDA tensors in the compact layout.
    Differentiable in every tensor argument."""
    return _Rollout.apply(G0, sl, u, v, w, (p, int(n_steps), precision, int(checkpoint)))


def _make_rollout():
    import torch

    class Rollout(torch.autograd.Function):
        @staticmethod
        def forward(ctx, G0, sl, u, v, w, spec):
            p, n_steps, precision, ckpt = spec
            for t in (G0, sl, u, v) + ((w,) if p.dim == 3 else ()):
                if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
                    raise ValueError("rollout wants contiguous float64 CUDA tensors")
            torch.cuda.current_stream().synchronize()
            s = lsgb.Solver(p, precision)
            s.set_fields(G0, u, v, w if p.dim == 3 else None, layout="compact")
            s.set_sl_field(sl, layout="compact")
            a = lsgb.Adjoint(s, ckpt)
            a.set_grads(sl=ctx.needs_input_grad[1], velocity=any(ctx.needs_input_grad[2:5]))
            a.forward(n_steps)
            out = torch.empty_like(G0)
            s.get_G(layout="compact", out=out)
            ctx.handles = (s, a)
            ctx.dim = p.dim
            return out

        @staticmethod
        def backward(ctx, gout):
            s, a = ctx.handles
            torch.cuda.current_stream().synchronize()
            a.backward(gout.contiguous(), layout="compact")
            names = ["G0", "sl", "u", "v", "w"]
            grads = []
            for q, name in enumerate(names):
                if ctx.needs_input_grad[q] and not (name == "w" and ctx.dim == 2):
                    t = torch.empty_like(gout)
                    a.grad(name, layout="compact", out=t)
                    grads.append(t)
                else:
                    grads.append(None)
            a.close()
            s.close()
            ctx.handles = None
            return (*grads, None)

    return Rollout


class _Lazy:
    def __init__(self):
        self._cls = None

    def apply(self, *args):
        if self._cls is None:
            self._cls = _make_rollout()
        return self._cls.apply(*args)


_Rollout = _Lazy()


def heaviside_loss(G, G_target, eps: float, dv: float):
    """torch form of the smoothed-Heaviside mismatch (same formula as
    lsgb_adjoint_loss)."""
    import torch
    h = 0.5 * (1.0 - torch.tanh(G / eps))
    ht = 0.5 * (1.0 - torch.tanh(G_target / eps))
    return 0.5 * torch.sum((h - ht) ** 2) * dv


# -- report -------------------------------------------------------------------
def report(n: int = 192, steps: int = 300, dirs: int = 32, checkpoint: int = 20, rel_step=1e-3,
           reinit: bool = True) -> dict:
    import torch  # noqa: F401  (CUDA context for the timing events)
    p, G0, u, v, w, sl, sl_t = workload(n, steps, reinit=reinit)
    out = {"n": n, "steps": steps, "checkpoint": checkpoint, "dt": p.dt, "dirs": dirs, "rel_step": rel_step,
           "reinit": reinit}
    # FP32 adjoint (the product form) and its cost against one plain forward
    p32 = Problem(p, G0, u, v, w, "f32", checkpoint)
    p32.a.set_grads(sl=True, velocity=False)
    p32.target(sl_t, steps)
    p32.run(sl, steps)
    p32.s.volume()
    t = time.perf_counter()
    p32.run(sl, steps)
    p32.s.volume()
    t_fwd = time.perf_counter() - t
    t = time.perf_counter()
    L32, g32 = p32.gradient(sl, steps)
    t_adj = time.perf_counter() - t
    out.update({"loss_f32": L32, "seconds_forward_f32": t_fwd, "seconds_forward_plus_backward_f32": t_adj,
                "adjoint_over_forward": t_adj / t_fwd})
    p32.close()
    # FP64 adjoint and the finite differences of the FP64 forward
    p64 = Problem(p, G0, u, v, w, "f64", checkpoint)
    p64.a.set_grads(sl=True, velocity=False)
    p64.target(sl_t, steps)
    t = time.perf_counter()
    L64, g64, rows = fd_check(p64, sl, steps, dirs, rel_step)
    out["seconds_fd_f64"] = time.perf_counter() - t
    p64.close()
    out.update({"loss_f64": L64,
                "grad_f32_vs_f64_rel_l2": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64)), "fd": rows})
    for rs in sorted({r["rel_step"] for r in rows}, reverse=True):
        rel = [r["rel_err"] for r in rows if r["rel_step"] == rs]
        out[f"fd_rel_err_max@{rs:g}"] = max(rel)
        out[f"fd_rel_err_median@{rs:g}"] = float(np.median(rel))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=192)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--dirs", type=int, default=32)
    ap.add_argument("--checkpoint", type=int, default=20)
    ap.add_argument("--rel-step", type=float, nargs="+", default=[1e-3])
    ap.add_argument("--no-reinit", action="store_true", help="drop HCR-2 (its crossing flags and stability "
                    "mask make the forward map discontinuous)")
    ap.add_argument("--json", default=None)
    ap.add_argument("--directional", action="store_true",
                    help="only the FP64 adjoint's directional derivatives and the loss")
    a = ap.parse_args()
    import __graft_entry__
    __graft_entry__.build_library()
    if a.directional:
        r = directional(a.n, a.steps, a.dirs, a.checkpoint)
        if a.json:
            with open(a.json, "w") as f:
                json.dump(r, f, indent=2)
        print(json.dumps(r))
        return
    r = report(a.n, a.steps, a.dirs, a.checkpoint, a.rel_step if len(a.rel_step) > 1 else a.rel_step[0],
               reinit=not a.no_reinit)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(r, f, indent=2)
    print(json.dumps({k: v for k, v in r.items() if k != "fd"}))


if __name__ == "__main__":
    main()
