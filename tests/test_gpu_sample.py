"""The sample surface on the GPU (lsgb_sample_*) against the committed
golden fixtures (made from the reference's compiled sources) and the oracle
port, bit for bit.  Needs a GB300."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def T(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def H(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("tag", ["24x20", "3x3"])
def test_sample_matches_golden(cuda, lsgb_mod, tag):
    from lsgb import sample as smp
    g = np.load(os.path.join(GOLDEN, f"golden_sample_{tag}.npz"))
    G, G0, u, v = g["G"], g["G0"], g["u"], g["v"]
    dx, dy, dt, sl = float(g["dx"]), float(g["dy"]), float(g["dt"]), float(g["S_L"])
    assert np.array_equal(H(smp.rhs(T(G), T(u), T(v), dx, dy, sl)), g["rhs"])
    assert np.array_equal(H(smp.rk3_step(T(G), T(u), T(v), dx, dy, dt, sl, T(G0))), g["rk3"])
    assert np.array_equal(H(smp.apply_periodic(T(G))), g["periodic"])
    assert np.array_equal(H(smp.apply_anchored_bc(T(G), T(G0))), g["anchored"])
    assert np.array_equal(H(smp.reinitialize(T(G), T(G0), dx, dy, 10)), g["reinit10"])
    assert np.array_equal(H(smp.first_order_upwind(T(G), T(u), T(v), dx, dy, dt, sl)), g["fou"])
    Gd = T(G)
    t = smp.run(Gd, T(G0), 25, dx, dy, [0], dt=dt, S_L=sl)
    assert np.array_equal(H(Gd), g["run25_f0"]) and t[0] == float(g["t25_f0"])


@pytest.mark.parametrize("nx,ny", [(64, 48), (37, 53), (3, 3), (4, 7), (200, 160)])
def test_sample_matches_port(cuda, lsgb_mod, port, nx, ny):
    from oracle import SampleOracle
    from lsgb import sample as smp
    so = SampleOracle("port")
    rng = np.random.default_rng(nx * 1000 + ny)
    G0 = smp.bunsen(nx, ny)
    dx, dy = smp.spacing(nx, ny)
    G = G0 + 1e-4 * rng.standard_normal(G0.shape)
    u = 0.3 * rng.standard_normal(G0.shape)
    v = 0.8 + 0.3 * rng.standard_normal(G0.shape)
    dt = 0.2 * min(dx, dy)
    assert np.array_equal(H(smp.rhs(T(G), T(u), T(v), dx, dy, 0.4)), so.rhs(G, u, v, dx, dy, 0.4))
    Gd = T(G)
    ref = G.copy()
    for _ in range(3):
        smp.rk3_step(Gd, T(u), T(v), dx, dy, dt, 0.4, T(G0))
        ref = so.rk3_step(ref, u, v, dx, dy, dt, 0.4, G0)
    assert np.array_equal(H(Gd), ref)
    for iters in (1, 4):
        assert np.array_equal(H(smp.reinitialize(T(G), T(G0), dx, dy, iters)),
                              so.reinitialize(G, G0, dx, dy, iters))
    # first-order upwind scheme: three steps in place, and a flat field (the |grad G| = 0 gate)
    Gd, ref = T(G), G.copy()
    for _ in range(3):
        smp.first_order_upwind(Gd, T(u), T(v), dx, dy, dt, 0.4)
        ref = so.first_order_upwind(ref, u, v, dx, dy, dt, 0.4)
    assert np.array_equal(H(Gd), ref)
    flat = np.ascontiguousarray(np.full_like(G, 0.25))
    assert np.array_equal(H(smp.first_order_upwind(T(flat), T(u), T(v), dx, dy, dt, 0.4)),
                          so.first_order_upwind(flat, u, v, dx, dy, dt, 0.4))


def test_frequency_sweep_matches_port_per_instance(cuda, lsgb_mod):
    """One call advances a stack of instances, each with its own forcing
    frequency and start time; every instance equals its own port run."""
    import torch
    from oracle import SampleOracle
    from lsgb import sample as smp
    so = SampleOracle("port")
    nx, ny = 48, 40
    G0 = smp.bunsen(nx, ny)
    dx, dy = smp.spacing(nx, ny)
    freqs = [5, 20, 50, 100, 200]
    t0 = [0.0, 1e-3, 0.0, 2.5e-4, 0.0]
    dt = 2e-4
    rng = np.random.default_rng(7)
    inits = [G0 + 1e-4 * rng.standard_normal(G0.shape) for _ in freqs]
    stack = torch.stack([T(a) for a in inits]).contiguous()
    t = smp.run(stack, T(G0), 40, dx, dy, freqs, t=t0, dt=dt)
    t = smp.run(stack, T(G0), 13, dx, dy, freqs, t=t, dt=dt)  # resume from the returned times
    for q, f in enumerate(freqs):
        ref, tr = so.run(inits[q], G0, 40, dx, dy, dt, smp.SL, smp.U0, smp.V0, smp.EPS_U, smp.EPS_V, f, t0[q])
        ref, tr = so.run(ref, G0, 13, dx, dy, dt, smp.SL, smp.U0, smp.V0, smp.EPS_U, smp.EPS_V, f, tr)
        assert np.array_equal(H(stack[q]), ref), f
        assert t[q] == tr


def test_sample_argument_errors(cuda, lsgb_mod):
    import torch
    from lsgb import sample as smp
    G = torch.zeros((2 + 6, 5 + 6), dtype=torch.float64, device="cuda")
    with pytest.raises(lsgb_mod.LsgbError):
        smp.apply_periodic(G)  # ny = 2 < 3
    G = torch.zeros((9, 9), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        smp.apply_periodic(G.float())
    with pytest.raises(lsgb_mod.LsgbError):
        smp.reinitialize(G, G, 0.0, 1.0, 2)
