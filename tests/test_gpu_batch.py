"""Batched instances and tile shapes (needs a GB300).

* A batch of uneven 2D and 3D instances advanced with captured-and-replayed
  CUDA graphs gives, per instance, exactly the single-instance result.
* Every tile shape of the FP32 kernels gives bit-identical fields (the
  autotuner only changes speed).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(2, (40, 40, 1)), (2, (67, 53, 1)), (2, (130, 96, 1)), (3, (20, 20, 20)),
         (3, (33, 17, 40)), (3, (48, 40, 70)), (2, (64, 64, 1)), (3, (32, 32, 32))]


def instance(lsgb, syn, dim, n, idx, precision, iters=2):
    rng = np.random.default_rng(4000 + idx)
    if dim == 3:
        wl = syn.sphere_config(4, n[0], 8, float(rng.uniform(0.05, 0.3)), instance=idx,
                               r0=float(rng.uniform(0.15, 0.3)), center=tuple(rng.uniform(0.35, 0.65, 3)))
        wl.n = n
    else:
        wl = syn.Workload(dim=2, n=n[:2], s_l=float(rng.uniform(0.05, 0.3)),
                          center=(*rng.uniform(0.35, 0.65, 2), 0.0), r0=float(rng.uniform(0.15, 0.3)))
        ks, cs, ph = syn.draw_modes(rng, 2, 8)
        wl.vel_k, wl.vel_c, wl.vel_phase = ks, cs, ph
    G, u, v, w = syn.host_fields(wl)
    dt = syn.cfl_dt(wl, u, v, w, 0.5)
    nz = n[2] if dim == 3 else 1
    p = lsgb.params(dim, n[0], n[1], nz, dx=1 / n[0], dy=1 / n[1], dz=1 / nz if dim == 3 else 1 / n[0],
                    s_l=wl.s_l, dt=dt, enable_reinit=True, reinit_interval=5, reinit_iterations=iters)
    return p, (G, u, v, w)


@pytest.mark.parametrize("precision,mode,iters", [("f32", "grouped", 2), ("f32", "grouped", 3), ("f32", "lanes", 2),
                                                  ("f64", "lanes", 2)])
def test_batch_matches_single_runs(cuda, lsgb_mod, precision, mode, iters):
    """Grouped form: one launch per RK3 stage and per pseudo-step for all 3D
    instances and one for all 2D ones, plus a copy back per dimensionality
    when the pseudo-step count is odd (an even count ends in G), so a
    captured period of 5 steps + HCR-2 holds 5 x 6 + 2 x 2 = 34 kernels with
    2 pseudo-steps and 5 x 6 + 3 x 2 + 2 = 38 with 3, whatever the number of
    instances."""
    from lsgb import synthetic as syn
    cases = [instance(lsgb_mod, syn, d, n, i, precision, iters) for i, (d, n) in enumerate(SIZES)]
    steps = 12  # step 0 direct, a captured period, a replayed period, one direct step
    with lsgb_mod.Batch(precision, lanes=4) as b:
        b.set_mode(mode)
        for p, f in cases:
            s = b.add(p)
            s.set_fields(*f)
        if precision == "f32":
            b.autotune()
        assert b.mode == mode
        b.advance(steps)
        b.sync()
        replays, kernels = b.stats()
        got = [s.get_G() for s in b.instances]
        tiles = [s.get_tile() for s in b.instances]
        assert all(s.step == steps for s in b.instances)
    assert replays == 2 and kernels > 0
    if mode == "grouped":
        assert kernels == 5 * 6 + iters * 2 + (2 if iters % 2 else 0)
    for (p, f), g, tile in zip(cases, got, tiles):
        with lsgb_mod.Solver(p, precision) as s:
            s.set_fields(*f)
            s.advance(steps)
            ref = s.get_G()
        assert np.array_equal(g, ref), (p.dim, p.nx, tile)


def test_tile_shapes_are_bit_identical(cuda, lsgb_mod):
    """Explicit shapes and the default (0) agree bit for bit; the 3D cases
    cover the bulk-tensor staging (nx % 4 == 0) and the cp.async staging."""
    from lsgb import synthetic as syn
    for dim, n in [(3, (36, 20, 70)), (3, (37, 21, 30)), (2, (70, 45, 1))]:
        p, f = instance(lsgb_mod, syn, dim, n, 7, "f32")
        outs = []
        tiles = [16, 32, 64] if dim == 3 else [32, 16]
        for tile in [0] + tiles:
            with lsgb_mod.Solver(p, "f32") as s:
                s.set_fields(*f)
                s.set_tile(tile)
                s.advance(7)
                outs.append(s.get_G())
        for o in outs[1:]:
            assert np.array_equal(o, outs[0])
        with lsgb_mod.Solver(p, "f32") as s:
            s.set_fields(*f)
            best, ms = s.autotune()
            assert best in tiles and ms > 0
            with pytest.raises(lsgb_mod.LsgbError):
                s.set_tile(5)
