"""Host-side helpers of the package (workload generators, report metrics):
CPU only, no GPU and no compute through the library."""
import math

import numpy as np


def test_fourier_field_is_seeded_and_normalised():
    from lsgb import adjoint as adj
    f = adj.fourier_field((12, 10, 8), 5)
    assert f.shape == (8, 10, 12)
    assert abs(np.abs(f).max() - 1.0) < 1e-12
    assert np.array_equal(f, adj.fourier_field((12, 10, 8), 5))
    assert not np.array_equal(f, adj.fourier_field((12, 10, 8), 6))
    sl = adj.sl_field((12, 10, 8), 5)
    assert 0.1 - 1e-12 <= sl.min() and sl.max() <= 0.2 + 1e-12


def test_adjoint_workload_shapes():
    from lsgb import adjoint as adj
    p, G0, u, v, w, sl, sl_t = adj.workload(16, 30)
    assert G0.shape == u.shape == w.shape == sl.shape == (16, 16, 16)
    assert p.dt > 0 and p.enable_reinit == 1 and p.reinit_interval == 10
    speed = float((np.abs(u) + np.abs(v) + np.abs(w)).max()) + float(max(sl.max(), sl_t.max()))
    assert math.isclose(p.dt, 0.5 / 16 / speed, rel_tol=1e-12)
    p2, G2, u2, v2, w2, *_ = adj.workload(24, 10, dim=2)
    assert G2.shape == (24, 24) and w2 is None and p2.dim == 2


def test_crossing_error_normal_displacement():
    from lsgb import precision as P
    n = 32
    dx = 1.0 / n
    x = np.arange(n) / n
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    g = np.sqrt((xx - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2) - 0.3
    cmax, cmean, count, nmax, nmean = P.crossing_error(g + 1e-6, g, dx)
    assert count > 1000
    # a uniform shift of 1e-6 moves the front by 1e-6 along the normal
    assert abs(nmean - 1e-6 / dx) < 0.05 * 1e-6 / dx
    assert cmax >= nmax  # grazing edges inflate the along-edge shift


def test_config4_instances():
    from lsgb import synthetic as syn
    wls = syn.config4()
    assert len(wls) == 96
    d2 = [w for w in wls if w.dim == 2]
    d3 = [w for w in wls if w.dim == 3]
    assert len(d2) == 48 and len(d3) == 48
    assert all(64 <= w.n[0] <= 1024 for w in d2) and all(32 <= w.n[0] <= 192 for w in d3)
    assert all(0.05 <= w.s_l <= 0.3 for w in wls)


def test_bunsen_initial_field():
    from lsgb import sample as smp
    nx, ny = 40, 30
    G = smp.bunsen(nx, ny)
    dx, dy = smp.spacing(nx, ny)
    assert G.shape == (ny + 6, nx + 6)
    assert math.isclose(dx, 0.02 / 39) and math.isclose(dy, 0.02 / 29)
    slope = math.tan(math.radians(60.0))
    for j, i in ((3, 3), (10, 20), (25, 40)):
        x, y = (i - 3) * dx, (j - 3) * dy
        d = slope * (x - 0.005) - y if x < 0.01 else -slope * (x - 0.015) - y
        assert math.isclose(G[j, i], -d, rel_tol=0, abs_tol=1e-15)
