"""Seeded synthetic workloads of the benchmark configurations.

No dataset is involved: every input is generated from a seed.  The mode
tables are drawn here with numpy's PCG64 (``default_rng``), seed
``20261203 + 1000 * config + instance``; the same table drives

* :func:`host_fields` -- the fields evaluated in numpy FP64 on the host (tests,
  and the CPU baselines on the full benchmark grid), and
* :func:`to_device_desc` -- the ``lsgb_synth`` descriptor the device generator
  (csrc/synth.cu) evaluates in FP64 for the large grids.

Fields (cell centres x_i = i * dx on the periodic unit box):
  G0 = |x - c| - (r0 + sum_m a_m Y_m(theta, phi))   sphere with l <= 4 modes
  G0 = |x - c| - r0                                 circle (2D)
  u  = curl A,  A = sum_m a_m sin(2 pi k_m . x + phase_m),  0 < |k_m| <= kmax,
       a_m ~ N(0, 1)^3, phase ~ U(0, 2 pi); 2D: stream function, u = (psi_y, -psi_x).
  The velocity is scaled so that max |u|_2 = 1 over the grid.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SEED_BASE = 20261203


def seed_for(config: int, instance: int = 0) -> int:
    return SEED_BASE + 1000 * config + instance


def _assoc_legendre(l: int, m: int, x):
    """P_l^m(x), 0 <= m <= l, no Condon-Shortley phase (same recursion as synth.cu)."""
    x = np.asarray(x, dtype=np.float64)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    pmm = np.ones_like(x)
    for q in range(1, m + 1):
        pmm = pmm * ((2.0 * q - 1.0) * s)
    if l == m:
        return pmm
    pm1 = x * (2.0 * m + 1.0) * pmm
    if l == m + 1:
        return pm1
    pl = pm1
    for ll in range(m + 2, l + 1):
        pl = (x * (2.0 * ll - 1.0) * pm1 - (ll + m - 1.0) * pmm) / (ll - m)
        pmm, pm1 = pm1, pl
    return pl


def _legendre_max(l: int, m: int) -> float:
    xs = np.linspace(-1.0, 1.0, 20001)
    return float(np.max(np.abs(_assoc_legendre(l, m, xs))))


@dataclass
class Workload:
    """One synthetic instance: grid, physics and mode table."""

    dim: int
    n: tuple
    s_l: float
    center: tuple = (0.5, 0.5, 0.5)
    r0: float = 0.2
    shape_l: list = field(default_factory=list)
    shape_m: list = field(default_factory=list)
    shape_amp: list = field(default_factory=list)   # already normalised
    vel_k: list = field(default_factory=list)
    vel_c: list = field(default_factory=list)       # 2 pi k x a  (2D: 2 pi a (k_y, -k_x))
    vel_phase: list = field(default_factory=list)
    uniform_velocity: tuple | None = None           # config 1: u = (1, 0)

    @property
    def spacing(self):
        return tuple(1.0 / q for q in self.n)


def draw_modes(rng: np.random.Generator, dim: int, n_vel: int, kmax: int = 4):
    ks, cs, ph = [], [], []
    while len(ks) < n_vel:
        k = rng.integers(-kmax, kmax + 1, size=dim)
        r2 = int(np.sum(k * k))
        if r2 == 0 or r2 > kmax * kmax:
            continue
        if dim == 3:
            a = rng.standard_normal(3)
            c = 2.0 * math.pi * np.cross(k.astype(np.float64), a)
            ks.append([float(k[0]), float(k[1]), float(k[2])])
        else:
            a = rng.standard_normal()
            c = 2.0 * math.pi * a * np.array([k[1], -k[0], 0.0], dtype=np.float64)
            ks.append([float(k[0]), float(k[1]), 0.0])
        cs.append([float(c[0]), float(c[1]), float(c[2])])
        ph.append(float(rng.uniform(0.0, 2.0 * math.pi)))
    return ks, cs, ph


def draw_shape(rng: np.random.Generator, n_modes: int, amp: float = 0.02):
    ls, ms, amps = [], [], []
    for _ in range(n_modes):
        l = int(rng.integers(1, 5))
        m = int(rng.integers(-l, l + 1))
        a = float(rng.uniform(-amp, amp))
        ls.append(l)
        ms.append(m)
        amps.append(a / _legendre_max(l, abs(m)))
    return ls, ms, amps


def config1(n: int = 128) -> Workload:
    """2D plain FP64: circle r = 0.25 at (0.5, 0.5), u = (1, 0), S_L = 0.1."""
    return Workload(dim=2, n=(n, n), s_l=0.1, center=(0.5, 0.5, 0.0), r0=0.25,
                    uniform_velocity=(1.0, 0.0))


def sphere_config(config: int, n: int, n_vel: int, s_l: float, instance: int = 0,
                  n_shape: int = 8, r0: float = 0.2, center=(0.5, 0.5, 0.5)) -> Workload:
    """Configs 2/3: perturbed sphere + curl of a random vector potential."""
    rng = np.random.default_rng(seed_for(config, instance))
    ls, ms, amps = draw_shape(rng, n_shape)
    ks, cs, ph = draw_modes(rng, 3, n_vel)
    return Workload(dim=3, n=(n, n, n), s_l=s_l, center=tuple(center), r0=r0, shape_l=ls,
                    shape_m=ms, shape_amp=amps, vel_k=ks, vel_c=cs, vel_phase=ph)


def config2(n: int = 256) -> Workload:
    return sphere_config(2, n, 16, 0.2)


def config3(n: int = 512) -> Workload:
    return sphere_config(3, n, 24, 0.2)


def _coords(wl: Workload, lo: int, hi: int):
    """Cell-centre coordinates of interior slab [lo, hi) along the slowest
    axis (z in 3D, y in 2D)."""
    axes = [np.arange(q, dtype=np.float64) / q for q in wl.n]
    if wl.dim == 3:
        z, y, x = np.meshgrid(axes[2][lo:hi], axes[1], axes[0], indexing="ij")
        return x, y, z
    y, x = np.meshgrid(axes[1][lo:hi], axes[0], indexing="ij")
    return x, y, np.zeros_like(x)


def _slab(wl: Workload, lo: int, hi: int):
    """(G, u, v, w) of interior slab [lo, hi), velocity not yet normalised."""
    x, y, z = _coords(wl, lo, hi)
    px, py = x - wl.center[0], y - wl.center[1]
    pz = z - wl.center[2] if wl.dim == 3 else np.zeros_like(x)
    rad = np.sqrt(px * px + py * py + pz * pz)
    radius = np.full_like(rad, wl.r0)
    if wl.dim == 3 and wl.shape_l:
        with np.errstate(invalid="ignore", divide="ignore"):
            ct = np.where(rad > 0, pz / np.where(rad > 0, rad, 1.0), 0.0)
        ph = np.arctan2(py, px)
        for l, m, a in zip(wl.shape_l, wl.shape_m, wl.shape_amp):
            am = abs(m)
            trig = np.cos(am * ph) if m >= 0 else np.sin(am * ph)
            radius = radius + np.where(rad > 0, a * _assoc_legendre(l, am, ct) * trig, 0.0)
    G = rad - radius
    if wl.uniform_velocity is not None:
        u = np.full_like(G, wl.uniform_velocity[0])
        v = np.full_like(G, wl.uniform_velocity[1])
        w = np.zeros_like(G)
    else:
        u = np.zeros_like(G)
        v = np.zeros_like(G)
        w = np.zeros_like(G)
        for k, c, phs in zip(wl.vel_k, wl.vel_c, wl.vel_phase):
            th = 2.0 * math.pi * (k[0] * x + k[1] * y + k[2] * z) + phs
            cs = np.cos(th)
            u += c[0] * cs
            v += c[1] * cs
            w += c[2] * cs
    return G, u, v, w


def _wrap_ghosts(a: np.ndarray, g: int = 3):
    """Fill the g-deep ghost layers of every axis with periodic images, in
    place (the same values as np.pad(interior, g, mode="wrap"))."""
    for ax in range(a.ndim - 1, -1, -1):
        n = a.shape[ax] - 2 * g
        idx = lambda s: tuple(s if d == ax else slice(None) for d in range(a.ndim))
        a[idx(slice(0, g))] = a[idx(slice(n, n + g))]
        a[idx(slice(n + g, n + 2 * g))] = a[idx(slice(g, 2 * g))]


def host_fields(wl: Workload, normalise: bool = True, threads: int | None = None):
    """(G, u, v, w) float64 in the ghosted layout, ghosts = periodic images.
    w is None in 2D.  Evaluated at interior cells in slabs along the slowest
    axis (in parallel threads; every value is an element-wise expression, so
    the slab size does not change a bit), then wrapped."""
    import concurrent.futures as cf
    import os

    shape = tuple(q + 6 for q in reversed(wl.n))
    G, u, v = (np.empty(shape) for _ in range(3))
    w = np.empty(shape) if wl.dim == 3 else None
    nslow = wl.n[-1]
    per_plane = int(np.prod(wl.n[:-1]))
    step = max(1, min(nslow, (1 << 21) // max(per_plane, 1)))
    inner = (slice(3, -3),) * (wl.dim - 1)

    def work(lo):
        hi = min(nslow, lo + step)
        g, a, b, c = _slab(wl, lo, hi)
        sl = (slice(3 + lo, 3 + hi),) + inner
        G[sl], u[sl], v[sl] = g, a, b
        if w is not None:
            w[sl] = c
        sp = np.sqrt(a * a + b * b + (c * c if wl.dim == 3 else 0.0))
        return float(sp.max())

    nthr = threads or min(16, os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=nthr) as ex:
        m = max(ex.map(work, range(0, nslow, step)))
    if wl.uniform_velocity is None and normalise and m > 0:
        for a in (u, v, w):
            if a is not None:
                a /= m
    for a in (G, u, v, w):
        if a is not None:
            _wrap_ghosts(a)
    return G, u, v, w


def to_device_desc(wl: Workload, normalise: bool = True):
    """The lsgb_synth descriptor of the workload (device generator)."""
    from . import Synth, MAX_MODES

    d = Synth()
    for q in range(3):
        d.center[q] = wl.center[q] if q < len(wl.center) else 0.0
    d.r0 = wl.r0
    if len(wl.shape_l) > MAX_MODES or len(wl.vel_k) > MAX_MODES:
        raise ValueError("too many modes")
    d.n_shape_modes = len(wl.shape_l)
    for q, (l, m, a) in enumerate(zip(wl.shape_l, wl.shape_m, wl.shape_amp)):
        d.shape_l[q], d.shape_m[q], d.shape_amp[q] = l, m, a
    if wl.uniform_velocity is not None:
        # a single k = 0 mode with phase 0 gives cos(0) = 1 times c
        d.n_vel_modes = 1
        d.vel_c[0][0], d.vel_c[0][1], d.vel_c[0][2] = wl.uniform_velocity[0], wl.uniform_velocity[1], 0.0
        d.vel_scale = 1.0
        return d
    d.n_vel_modes = len(wl.vel_k)
    for q, (k, c, ph) in enumerate(zip(wl.vel_k, wl.vel_c, wl.vel_phase)):
        for a in range(3):
            d.vel_k[q][a] = k[a]
            d.vel_c[q][a] = c[a]
        d.vel_phase[q] = ph
    d.vel_scale = 0.0 if normalise else 1.0
    return d


def cfl_dt(wl: Workload, u, v, w, cfl: float, epsilon: float = 1e-10) -> float:
    """CFL step from the field max of |u|+|v|+|w| (calculateTimeStep form,
    Local_code/level-set_MPI_3D/include/config.h:272-293)."""
    sl = (slice(3, -3),) * wl.dim
    s = np.abs(u[sl]) + np.abs(v[sl])
    if wl.dim == 3:
        s = s + np.abs(w[sl])
    speed = float(s.max()) + wl.s_l
    if speed < epsilon:
        speed = 2.0
    return cfl * min(wl.spacing) / speed


def config4(n2d: int = 48, n3d: int = 48, n_vel: int = 8):
    """Batched form: n2d 2D instances with N = round(exp(U(ln 64, ln 1024)))
    per axis and n3d 3D instances with N = round(exp(U(ln 32, ln 192))); a
    circle / sphere of radius U(0.15, 0.3) at a random centre, an n_vel-mode
    random divergence-free velocity and S_L ~ U(0.05, 0.3) per instance."""
    out = []
    for j in range(n2d + n3d):
        rng = np.random.default_rng(seed_for(4, j))
        dim = 2 if j < n2d else 3
        lo, hi = (64, 1024) if dim == 2 else (32, 192)
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        r0 = float(rng.uniform(0.15, 0.3))
        c = rng.uniform(0.3, 0.7, 3)
        s_l = float(rng.uniform(0.05, 0.3))
        ks, cs, ph = draw_modes(rng, dim, n_vel)
        out.append(Workload(dim=dim, n=(n,) * dim, s_l=s_l, center=(float(c[0]), float(c[1]), float(c[2]) if dim == 3 else 0.0),
                            r0=r0, vel_k=ks, vel_c=cs, vel_phase=ph))
    return out


# ---- the reference's 2D known-answer case -----------------------------------
ZALESAK_T_FINAL = 6.283185  # T_FINAL, Local_code/level-set_MPI_2D/include/config.h:65


def zalesak_fields(n: int):
    """(G0, u, v) of the reference's Zalesak case on an n x n grid of [0,1]^2
    (dx = 1/(n-1)), ghosted (n+6, n+6) float64 arrays with the same rounded
    operations as initZalesakTestCase (Local_code/level-set_MPI_2D/include/
    initial_conditions.h:91-125, 209-227, 260-272; coordinates config.h:281-294):
    slotted disk (0.5, 0.75), r = 0.15, slot 0.05 x 0.25, rotated about
    (0.5, 0.5) at omega = 2 pi / T_FINAL.  Ghost values follow the same
    formula (the solvers read only interior cells of the inputs).  Returns
    also dx and the CFL time step (0.2 dx / |u_const|, u_const = 1)."""
    dx = (1.0 - 0.0) / (n - 1)
    idx = (np.arange(n + 6) - 3).astype(np.float64)
    x1 = 0.0 + idx * dx
    y1 = 0.0 + idx * dx
    y, x = np.meshgrid(y1, x1, indexing="ij")
    cx, cy, r, sw, sln = 0.5, 0.75, 0.15, 0.05, 0.25
    ddx = x - cx
    ddy = y - cy
    dist_disk = np.sqrt(ddx * ddx + ddy * ddy) - r
    half = sw / 2.0
    bottom = cy - r
    top = bottom + sln
    sdx = np.abs(x - cx) - half
    sdy = np.fmax(bottom - y, y - top)
    dist_slot = np.where((sdx < 0.0) & (sdy < 0.0), np.fmax(sdx, sdy),
                         np.where(sdx < 0.0, sdy, np.where(sdy < 0.0, sdx, np.sqrt(sdx * sdx + sdy * sdy))))
    G = np.fmax(dist_disk, -dist_slot)
    omega = 2.0 * math.pi / ZALESAK_T_FINAL
    u = -omega * (y - 0.5)
    v = omega * (x - 0.5)
    dt = 0.2 * min(dx, dx) / max(abs(1.0) + abs(0.0) + 0.0, 1e-10)
    return np.ascontiguousarray(G), np.ascontiguousarray(u), np.ascontiguousarray(v), dx, dt
