"""analyze_error.m diagnostics as a device reduction (needs a GB300), against
a numpy statement of the same definitions on periodic grids."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def np_diagnostics(G, R, h):
    """The quantities of lsgb_diagnostics from compact periodic arrays
    (axis order z, y, x / y, x; h = spacing per axis in x, y, z order)."""
    dim = G.ndim
    dv = float(np.prod(h[:dim]))
    d = G - R

    def grad(f):
        s = 0.0
        for ax in range(dim):
            a = dim - 1 - ax  # numpy axis of spatial axis ax
            s = s + ((np.roll(f, -1, a) - np.roll(f, 1, a)) / (2 * h[ax])) ** 2
        return np.sqrt(s)

    def H(phi, eps):
        out = np.where(phi > eps, 1.0, 0.0)
        m = np.abs(phi) <= eps
        out[m] = 0.5 * (1 + phi[m] / eps + np.sin(np.pi * phi[m] / eps) / np.pi)
        return out

    gG, gR = grad(G), grad(R)
    band = np.abs(G) < 3 * h[0]
    dists = []
    for ax in range(dim):
        a = dim - 1 - ax
        for p, o, go in ((G, R, gR), (R, G, gG)):
            p1, o1, g1 = np.roll(p, -1, a), np.roll(o, -1, a), np.roll(go, -1, a)
            m = p * p1 < 0
            t = p[m] / (p[m] - p1[m])
            ov = o[m] + t * (o1[m] - o[m])
            gp = go[m] + t * (g1[m] - go[m])
            dists.append(np.abs(ov) / gp)
    dists = np.concatenate(dists)
    gb = gG[band]
    return {"l2": np.sqrt(np.mean(d * d)), "linf": np.abs(d).max(),
            "l2_rel": np.sqrt(np.mean(d * d)) / np.sqrt(np.mean(R * R)),
            "volume": np.count_nonzero(G < 0) * dv, "volume_ref": np.count_nonzero(R < 0) * dv,
            "volume_smooth": H(-G, h[0]).sum() * dv, "volume_smooth_ref": H(-R, h[0]).sum() * dv,
            "grad_mean": gb.mean(), "grad_std": gb.std(ddof=1), "band_cells": int(band.sum()),
            "iface_mean": dists.mean(), "iface_max": dists.max(), "iface_points": dists.size}


@pytest.mark.parametrize("dim,n,prec", [(3, (40, 36, 44), "f64"), (3, (40, 36, 44), "f32"), (2, (96, 80, 1), "f64")])
def test_diagnostics_match_numpy(cuda, lsgb_mod, dim, n, prec):
    from lsgb import synthetic as syn
    if dim == 3:
        wl = syn.sphere_config(3, n[0], 8, 0.2)
    else:
        wl = syn.Workload(dim=2, n=n[:2], s_l=0.1, center=(0.5, 0.45, 0.0), r0=0.27)
        rng = np.random.default_rng(3)
        wl.vel_k, wl.vel_c, wl.vel_phase = syn.draw_modes(rng, 2, 6)
    wl.n = n[:dim]
    G, u, v, w = syn.host_fields(wl)
    h = (1 / n[0], 1 / n[1], 1 / n[2] if dim == 3 else 1 / n[0])
    p = lsgb_mod.params(dim, *n, dx=h[0], dy=h[1], dz=h[2], s_l=0.2, dt=1e-3, enable_reinit=True,
                        reinit_interval=3, reinit_iterations=2)
    with lsgb_mod.Solver(p, prec) as s:
        s.set_fields(G, u, v, w)
        s.advance(9)
        d = s.diagnostics(G)
        Gt = s.get_G(layout="compact")
    inner = (slice(3, -3),) * dim
    want = np_diagnostics(Gt, np.ascontiguousarray(G[inner]), h)
    for k, v in want.items():
        if k in ("band_cells", "iface_points"):
            assert d[k] == v, k
        else:
            assert d[k] == pytest.approx(v, rel=1e-9, abs=1e-15), k
