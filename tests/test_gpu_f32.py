"""Accuracy of the FP32-bulk form against the FP64 form (needs a GB300).

The FP32 path is not bit-exact by design.  Tolerances (stated here, checked
on every run):
  * smooth synthetic fields (the benchmark construction): after 20 RK3 steps
    with HCR-2 every 5, L_inf(G32 - G64) <= 2e-6 and, within 3 cells of the
    front, <= 1e-3 * dx (the FP32 form's bound on the zero-level-set error);
  * rough random fields (every upwind branch, non-smooth WENO weights):
    L_inf <= 5e-5 after 4 steps -- a kernel-logic check on ragged tiles,
    z-chunk seams, the 3-cell minimum and zero-gradient axes (y and z, or all
    three, with the bulk-tensor staging at nx = 36).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(lsgb, p, precision, n_steps, G, u, v, w, sl=None):
    with lsgb.Solver(p, precision) as s:
        s.set_fields(G, u, v, w)
        if sl is not None:
            s.set_sl_field(sl)
        s.advance(n_steps)
        return s.get_G(layout="compact")


@pytest.mark.parametrize("n", [(40, 36, 70), (64, 64, 64), (33, 17, 9)])
def test_f32_smooth_fields_vs_f64(cuda, lsgb_mod, n):
    from lsgb import synthetic as syn
    wl = syn.sphere_config(3, n[0], 24, 0.2)
    wl.n = n
    G, u, v, w = syn.host_fields(wl)
    dt = syn.cfl_dt(wl, u, v, w, 0.5)
    p = lsgb_mod.params(3, *n, dx=1 / n[0], dy=1 / n[1], dz=1 / n[2], s_l=0.2, dt=dt,
                        enable_reinit=True, reinit_interval=5, reinit_iterations=2)
    g64 = run(lsgb_mod, p, "f64", 20, G, u, v, w)
    g32 = run(lsgb_mod, p, "f32", 20, G, u, v, w)
    d = np.abs(g32 - g64)
    dx = 1.0 / min(n)
    band = np.abs(g64) < 3 * dx
    print(f"n={n}: linf={d.max():.3e} band3={d[band].max():.3e} ({d[band].max() / dx:.3e} dx)")
    assert d.max() <= 2e-6
    assert d[band].max() <= 1e-3 * dx


@pytest.mark.parametrize("n,bc", [((37, 19, 70), 0), ((33, 9, 5), 0), ((3, 3, 3), 0),
                                  ((35, 11, 66), 1), ((64, 16, 128), 0), ((36, 21, 33), 2)])
def test_f32_rough_fields_vs_f64(cuda, lsgb_mod, n, bc):
    rng = np.random.default_rng(sum(n) + bc)
    shape = tuple(q + 6 for q in reversed(n))
    zz, yy, xx = np.meshgrid(*[(np.arange(s) - 3) / q for s, q in zip(shape, reversed(n))], indexing="ij")
    G = np.sqrt((xx - .5) ** 2 + (yy - .45) ** 2 + (zz - .55) ** 2) - 0.3 + 0.02 * rng.standard_normal(shape)
    u, v, w = (rng.standard_normal(shape) for _ in range(3))
    sl = np.abs(rng.standard_normal(shape)) * 0.2
    # bc: 0 periodic, 1 zero-gradient in y and z, 2 zero-gradient on every axis
    p = lsgb_mod.params(3, *n, s_l=0.15, dt=2e-4, enable_reinit=True, reinit_interval=2,
                        reinit_iterations=2, bc_x=int(bc == 2), bc_y=int(bc > 0), bc_z=int(bc > 0))
    for field in (None, sl):
        g64 = run(lsgb_mod, p, "f64", 4, G, u, v, w, field)
        g32 = run(lsgb_mod, p, "f32", 4, G, u, v, w, field)
        err = float(np.abs(g32 - g64).max())
        print(f"n={n} bc={bc} sl_field={field is not None}: linf={err:.3e}")
        assert err <= 5e-5


def test_f32_single_stage_matches_f64(cuda, lsgb_mod):
    """One step with S_L = 0 on a smooth field: FP32 within 1e-6 of FP64."""
    from lsgb import synthetic as syn
    wl = syn.sphere_config(2, 48, 16, 0.0)
    G, u, v, w = syn.host_fields(wl)
    p = lsgb_mod.params(3, 48, 48, 48, s_l=0.0, dt=syn.cfl_dt(wl, u, v, w, 0.5))
    err = float(np.abs(run(lsgb_mod, p, "f32", 1, G, u, v, w) - run(lsgb_mod, p, "f64", 1, G, u, v, w)).max())
    print(f"single step linf={err:.3e}")
    assert err <= 1e-6


@pytest.mark.parametrize("n,bc", [((96, 70), 0), ((37, 21), 1), ((3, 3), 0), ((65, 33), 1)])
def test_f32_2d_vs_f64(cuda, lsgb_mod, n, bc):
    """2D FP32 stage kernel (row-pair tiles) against the FP64 form on rough
    random fields: ragged tiles, the 3-cell minimum, periodic or
    zero-gradient Y, per-cell S_L; L_inf <= 5e-5 after 4 steps."""
    rng = np.random.default_rng(n[0] * 7 + n[1] + bc)
    shape = (n[1] + 6, n[0] + 6)
    yy, xx = np.meshgrid(*[(np.arange(s) - 3) / q for s, q in zip(shape, (n[1], n[0]))], indexing="ij")
    G = np.sqrt((xx - .5) ** 2 + (yy - .45) ** 2) - 0.3 + 0.02 * rng.standard_normal(shape)
    u, v = (rng.standard_normal(shape) for _ in range(2))
    sl = np.abs(rng.standard_normal(shape)) * 0.2
    p = lsgb_mod.params(2, n[0], n[1], 1, s_l=0.15, dt=2e-4, enable_reinit=True, reinit_interval=2,
                        reinit_iterations=2, bc_y=bc)
    for field in (None, sl):
        g64 = run(lsgb_mod, p, "f64", 4, G, u, v, None, field)
        g32 = run(lsgb_mod, p, "f32", 4, G, u, v, None, field)
        err = float(np.abs(g32 - g64).max())
        print(f"2D n={n} bc={bc} sl_field={field is not None}: linf={err:.3e}")
        assert err <= 5e-5


def test_deformation_velocity_f32_vs_f64(cuda, lsgb_mod):
    """The on-device deformation vortex (computeDeformationVelocity,
    Local_code/level-set_MPI_3D/include/initial_conditions.h:232-247): the
    FP64 solver's field is the formula at x_i = i dx (numpy's sines, to 1e-15
    of max|u|); the FP32 solver forms the products in FP32 and stays within
    4 FP32 ulps of max|u| of the FP64 field.  Ragged sizes, unequal spacing."""
    n = (37, 21, 30)
    h = (1 / 36, 1 / 20, 1 / 29)
    t, T = 0.37, 1.5
    p = lsgb_mod.params(3, *n, dx=h[0], dy=h[1], dz=h[2], dt=1e-3)
    out = {}
    for prec in ("f64", "f32"):
        with lsgb_mod.Solver(p, prec) as s:
            s.set_velocity_deformation(t, T)
            out[prec] = [s.get_field(f, layout="compact") for f in ("u", "v", "w")]
    z, y, x = np.meshgrid(*[np.arange(q) * hq for q, hq in zip(n[::-1], h[::-1])], indexing="ij")
    tf = np.cos(np.pi * t / T)
    s1 = [np.sin(np.pi * c) for c in (x, y, z)]
    s2 = [np.sin(2 * np.pi * c) for c in (x, y, z)]
    ref = [2 * s1[0] ** 2 * s2[1] * s2[2] * tf, -s2[0] * s1[1] ** 2 * s2[2] * tf, -s2[0] * s2[1] * s1[2] ** 2 * tf]
    for r, a64, a32 in zip(ref, out["f64"], out["f32"]):
        scale = np.abs(r).max()
        assert np.abs(a64 - r).max() <= 1e-15 * scale
        assert np.abs(a32 - a64).max() <= 4 * np.finfo(np.float32).eps * scale
