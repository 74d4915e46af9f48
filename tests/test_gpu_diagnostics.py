"""analyze_error.m diagnostics as a device reduction (needs a GB300), against
a numpy statement of the same definitions on periodic grids, including the
script's interface position error (Local_code/level-set_MPI_3D/scripts/
analyze_error.m:51-84) by brute-force nearest points."""
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


def np_contour_points(F, h):
    """The zero contour as analyze_error.m takes it from contourc: the linear-
    interpolation crossings on the grid edges between interior cells (no
    wrap-around edge), one point per edge whose values change sign (one < 0,
    the other >= 0), in coordinates (i dx, j dy, k dz).  Rows (x, y, z)."""
    dim = F.ndim
    out = []
    for ax in range(dim):  # spatial axis 0 = x = the last numpy axis
        a = dim - 1 - ax
        lo = tuple(slice(0, -1) if q == a else slice(None) for q in range(dim))
        hi = tuple(slice(1, None) if q == a else slice(None) for q in range(dim))
        p0, p1 = F[lo], F[hi]
        m = (p0 < 0) != (p1 < 0)
        idx = np.nonzero(m)
        t = p0[m] / (p0[m] - p1[m])
        cols = []
        for sp in range(3):
            if sp >= dim:
                cols.append(np.zeros(t.size))
                continue
            i = idx[dim - 1 - sp].astype(np.float64)
            cols.append((i + t) * h[sp] if sp == ax else i * h[sp])
        out.append(np.stack(cols, 1))
    return np.concatenate(out)


def np_interface_error(A, B):
    """analyze_error.m:62-77: nearest-point distances both ways (brute force),
    Hausdorff = the largest, mean over both sets together."""
    def nearest(P, Q):
        d = np.empty(len(P))
        for s in range(0, len(P), 128):
            e = Q[None, :, :] - P[s:s + 128, None, :]
            d2 = (e[..., 0] * e[..., 0] + e[..., 1] * e[..., 1]) + e[..., 2] * e[..., 2]
            d[s:s + 128] = np.sqrt(d2.min(1))
        return d
    da, db = nearest(A, B), nearest(B, A)
    return max(da.max(), db.max()), np.concatenate([da, db]).mean()


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
    # the script's interface position error: device bins vs brute force
    A = np_contour_points(Gt, h)
    B = np_contour_points(np.ascontiguousarray(G[inner]), h)
    haus, mean = np_interface_error(A, B)
    assert (d["contour_points"], d["contour_points_ref"]) == (len(A), len(B))
    assert d["contour_hausdorff"] == pytest.approx(haus, rel=1e-12)
    assert d["contour_mean"] == pytest.approx(mean, rel=1e-12)
    assert 0 < d["contour_mean"] <= d["contour_hausdorff"]


def test_contour_distance_far_apart_and_empty(cuda, lsgb_mod):
    """Two discs far apart (the search must widen past many empty bins), and a
    field without a zero contour (the script's "could not extract" case: NaN)."""
    n = 64
    h = 1.0 / n
    y, x = np.meshgrid(np.arange(n) * h, np.arange(n) * h, indexing="ij")
    G = np.sqrt((x - 0.2) ** 2 + (y - 0.25) ** 2) - 0.1
    R = np.sqrt((x - 0.75) ** 2 + (y - 0.7) ** 2) - 0.15
    p = lsgb_mod.params(2, n, n, 1)
    with lsgb_mod.Solver(p, "f64") as s:
        s.set_fields(np.ascontiguousarray(np.pad(G, 3, mode="wrap")), layout="ghosted")
        d = s.diagnostics(np.ascontiguousarray(R), layout="compact")
        haus, mean = np_interface_error(np_contour_points(G, (h, h)), np_contour_points(R, (h, h)))
        assert d["contour_hausdorff"] == pytest.approx(haus, rel=1e-12)
        assert d["contour_mean"] == pytest.approx(mean, rel=1e-12)
        assert d["contour_mean"] > 0.3
        d = s.diagnostics(np.ascontiguousarray(np.ones((n, n))), layout="compact")
        assert d["contour_points_ref"] == 0 and np.isnan(d["contour_hausdorff"]) and np.isnan(d["contour_mean"])
