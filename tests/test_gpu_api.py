"""Solver-handle plumbing on the GPU: layouts, host/device transfers, the
end-to-end host call, the device generator, argument checks."""
import numpy as np
import pytest

from oracle import Problem

pytestmark = pytest.mark.gpu


def test_layouts_and_memory_kinds_agree(cuda, lsgb_mod, port):
    import torch
    pb = Problem(nx=11, ny=9, nz=7, dim=3, s_l=0.1, dt=1e-3)
    p = lsgb_mod.params(3, 11, 9, 7, s_l=0.1, dt=1e-3)
    rng = np.random.default_rng(2)
    G = port.apply_bc(pb, rng.standard_normal(pb.shape) * 0.1)
    vel = [port.apply_bc(pb, rng.standard_normal(pb.shape)) for _ in range(3)]
    inner = (slice(3, -3),) * 3
    ref = port.run(pb, 3, G, *vel)
    with lsgb_mod.Solver(p, "f64") as s:
        # compact host upload, device ghosted download
        s.set_fields(*[np.ascontiguousarray(a[inner]) for a in (G, *vel)], layout="compact")
        s.advance(3)
        out_dev = torch.zeros(pb.shape, dtype=torch.float64, device="cuda")
        s.get_G(out=out_dev)
        torch.cuda.synchronize()
        assert np.array_equal(out_dev.cpu().numpy(), ref)
        assert np.array_equal(s.get_G(layout="compact"), ref[inner])
        # device ghosted upload
        s.set_fields(*[torch.from_numpy(a).cuda() for a in (G, *vel)])
        s.step = 0
        s.advance(3)
        assert np.array_equal(s.get_G(), ref)


def test_run_host_equals_stepwise(cuda, lsgb_mod):
    p = lsgb_mod.params(3, 12, 12, 12, s_l=0.2, dt=1e-3, enable_reinit=True, reinit_interval=2)
    rng = np.random.default_rng(4)
    G = rng.standard_normal(p.shape()) * 0.1
    vel = [rng.standard_normal(p.shape()) for _ in range(3)]
    for prec in ("f64", "f32"):
        with lsgb_mod.Solver(p, prec) as s:
            out = np.empty_like(G)
            s.run_host(G, *vel, 5, out)
        with lsgb_mod.Solver(p, prec) as s:
            s.set_fields(G, *vel)
            s.advance(5)
            assert np.array_equal(s.get_G(), out)


def test_device_generator_matches_host(cuda, lsgb_mod):
    from lsgb import synthetic as syn
    wl = syn.sphere_config(2, 20, 16, 0.2)
    G, u, v, w = syn.host_fields(wl)
    p = lsgb_mod.params(3, 20, 20, 20, s_l=0.2)
    with lsgb_mod.Solver(p, "f64") as s:
        s.synth(syn.to_device_desc(wl))
        Gd = s.get_G()
        assert np.abs(Gd - G).max() < 1e-12
        assert s.max_speed() == pytest.approx(float((np.abs(u) + np.abs(v) + np.abs(w)).max()), rel=1e-12)
    wl2 = syn.config1(32)
    G2, _, _, _ = syn.host_fields(wl2)
    with lsgb_mod.Solver(lsgb_mod.params(2, 32, 32, s_l=0.1), "f64") as s:
        s.synth(syn.to_device_desc(wl2))
        assert np.abs(s.get_G() - G2).max() < 1e-14
        assert s.max_speed() == 1.0


def test_compute_dt_uses_field_max(cuda, lsgb_mod):
    from lsgb import synthetic as syn
    wl = syn.sphere_config(2, 16, 8, 0.2)
    G, u, v, w = syn.host_fields(wl)
    p = lsgb_mod.params(3, 16, 16, 16, s_l=0.2)
    with lsgb_mod.Solver(p, "f64") as s:
        s.set_fields(G, u, v, w)
        dt = s.compute_dt(0.5)
        assert dt == pytest.approx(syn.cfl_dt(wl, u, v, w, 0.5), rel=1e-15)
        assert s.params().dt == dt


def test_bad_arguments_raise(cuda, lsgb_mod):
    import torch
    p = lsgb_mod.params(3, 8, 8, 8)
    host_arr = np.zeros(p.shape())
    d = torch.zeros(p.shape(), dtype=torch.float64, device="cuda")
    with pytest.raises(lsgb_mod.LsgbError, match="not device memory"):
        lsgb_mod.rk3_step_f64(p, host_arr, d, d.clone(), d.clone(), d, d, d)
    with pytest.raises(lsgb_mod.LsgbError, match="distinct"):
        lsgb_mod.rk3_step_f64(p, d, d, d.clone(), d.clone(), d, d, d)
    with lsgb_mod.Solver(p) as s:
        with pytest.raises(lsgb_mod.LsgbError, match="not set"):
            s.advance(1)
        with pytest.raises(lsgb_mod.LsgbError):
            s.synth(lsgb_mod.Synth(n_vel_modes=99))
