"""Discrete adjoint of the solver (needs a GB300).

Checks, with the tolerances stated per test:
  * FP64 adjoint vs central finite differences of the FP64 forward along
    smooth random directions in S_L, G0 and u (relative step 1e-6; the
    frozen upwind / Godunov / constraint choices do not flip at that step):
    relative error <= 1e-5, with periodic and zero-gradient axes;
  * the same directional derivative from finite differences of the oracle's
    forward (the CPU restatement of the reference) on the ghosted layout,
    3D periodic and 2D with the reference's zero-gradient y;
  * gradients are bit-identical for every checkpoint interval;
  * the FP32 adjoint against the FP64 adjoint: relative L2 <= 1e-3;
  * live deformation velocity: FD of the live forward, checkpoint
    independence and FP32 vs FP64;
  * the torch autograd Function gives the native gradients.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small(lsgb_mod, dim, bc=None):
    from lsgb import adjoint as adj
    n, steps = (20, 12) if dim == 3 else (40, 15)
    p, G0, u, v, w, sl, sl_t = adj.workload(n, steps, dim=dim, reinit_interval=5, bc=bc)
    return adj, p, steps, G0, u, v, w, sl, sl_t


ZG = "zero_gradient"
# (dim, boundary per axis): periodic everywhere; the reference 2D solver's
# default (periodic x, zero-gradient y); a 3D mix with clamped x and z
FD_CASES = [(3, None), (2, None), (2, ("periodic", ZG)), (3, (ZG, "periodic", ZG))]


def loss_of(prob, G0, u, sl, steps):
    prob.G0, prob.u = G0, u
    return prob.loss(sl, steps)


@pytest.mark.parametrize("dim,bc", FD_CASES, ids=["3d", "2d", "2d-zgy", "3d-zgxz"])
def test_adjoint_matches_fd_f64(cuda, lsgb_mod, dim, bc):
    adj, p, steps, G0, u, v, w, sl, sl_t = small(lsgb_mod, dim, bc)
    prob = adj.Problem(p, G0, u, v, w, "f64", checkpoint=4)
    try:
        prob.target(sl_t, steps)
        L, g_sl = prob.gradient(sl, steps)
        g_G0 = prob.a.grad("G0")
        g_u = prob.a.grad("u")
        assert L > 0 and np.isfinite(g_sl).all() and np.abs(g_sl).max() > 0
        checks = []
        for q in range(3):
            d = adj.fourier_field(sl.shape[::-1], 11 + q)
            d /= np.linalg.norm(d)
            h = 1e-6 * np.linalg.norm(sl)
            fd = (loss_of(prob, G0, u, sl + h * d, steps) - loss_of(prob, G0, u, sl - h * d, steps)) / (2 * h)
            checks.append(("sl", fd, float(np.sum(g_sl * d))))
        d = adj.fourier_field(sl.shape[::-1], 31)
        d /= np.linalg.norm(d)
        h = 1e-6 * np.linalg.norm(G0)
        fd = (loss_of(prob, G0 + h * d, u, sl, steps) - loss_of(prob, G0 - h * d, u, sl, steps)) / (2 * h)
        checks.append(("G0", fd, float(np.sum(g_G0 * d))))
        h = 1e-6 * np.linalg.norm(u)
        fd = (loss_of(prob, G0, u + h * d, sl, steps) - loss_of(prob, G0, u - h * d, sl, steps)) / (2 * h)
        checks.append(("u", fd, float(np.sum(g_u * d))))
        prob.G0, prob.u = G0, u
    finally:
        prob.close()
    for name, fd, ad in checks:
        print(f"dim={dim} bc={bc} {name}: fd={fd:.10e} adjoint={ad:.10e} rel={abs(fd - ad) / abs(fd):.2e}")
        assert abs(fd - ad) <= 1e-5 * abs(fd), (name, fd, ad)


def test_adjoint_matches_fd_of_oracle(cuda, lsgb_mod, port):
    from oracle import Problem as OProblem
    adj, p, steps, G0, u, v, w, sl, sl_t = small(lsgb_mod, 3)
    n = p.nx
    pb = OProblem(n, n, n, dt=p.dt, s_l=p.s_l, enable_reinit=True, reinit_interval=5, reinit_iterations=2)
    gh = lambda a: np.ascontiguousarray(np.pad(a, 3, mode="wrap"))
    eps, dv = 1.5 / n, 1.0 / n ** 3

    def oracle_loss(s_field, G_target):
        out = port.run(pb, steps, gh(G0), gh(u), gh(v), gh(w), sl=gh(s_field))[3:-3, 3:-3, 3:-3]
        h, ht = 0.5 * (1 - np.tanh(out / eps)), 0.5 * (1 - np.tanh(G_target / eps))
        return 0.5 * np.sum((h - ht) ** 2) * dv

    prob = adj.Problem(p, G0, u, v, w, "f64", checkpoint=5)
    try:
        gt = prob.target(sl_t, steps)
        _, g_sl = prob.gradient(sl, steps)
    finally:
        prob.close()
    for q in range(2):
        d = adj.fourier_field(sl.shape[::-1], 51 + q)
        d /= np.linalg.norm(d)
        h = 1e-6 * np.linalg.norm(sl)
        fd = (oracle_loss(sl + h * d, gt) - oracle_loss(sl - h * d, gt)) / (2 * h)
        ad = float(np.sum(g_sl * d))
        print(f"oracle fd={fd:.10e} adjoint={ad:.10e}")
        assert abs(fd - ad) <= 1e-5 * abs(fd)


def test_adjoint_matches_fd_of_oracle_2d_zero_gradient_y(cuda, lsgb_mod, port):
    """The reference 2D solver's boundaries (periodic x, zero-gradient y;
    Local_code/level-set_MPI_2D/include/boundary.h:217): the adjoint's
    directional derivative against finite differences of the oracle's 2D
    forward with HCR-2 on (relative error <= 1e-5)."""
    from oracle import Problem as OProblem
    adj, p, steps, G0, u, v, w, sl, sl_t = small(lsgb_mod, 2, ("periodic", ZG))
    n = p.nx
    pb = OProblem(n, n, dim=2, dt=p.dt, s_l=p.s_l, enable_reinit=True, reinit_interval=5, reinit_iterations=2,
                  periodic_y=False)

    def gh(a):  # ghosted copy: y edge-padded, x wrapped
        return np.ascontiguousarray(np.pad(np.pad(a, ((3, 3), (0, 0)), mode="edge"), ((0, 0), (3, 3)), mode="wrap"))

    eps, dv = 1.5 / n, 1.0 / n ** 2

    def oracle_loss(s_field, G_target):
        out = port.run(pb, steps, gh(G0), gh(u), gh(v), sl=gh(s_field))[3:-3, 3:-3]
        h, ht = 0.5 * (1 - np.tanh(out / eps)), 0.5 * (1 - np.tanh(G_target / eps))
        return 0.5 * np.sum((h - ht) ** 2) * dv

    prob = adj.Problem(p, G0, u, v, w, "f64", checkpoint=4)
    try:
        gt = prob.target(sl_t, steps)
        _, g_sl = prob.gradient(sl, steps)
    finally:
        prob.close()
    for q in range(2):
        d = adj.fourier_field(sl.shape[::-1], 61 + q)
        d /= np.linalg.norm(d)
        h = 1e-6 * np.linalg.norm(sl)
        fd = (oracle_loss(sl + h * d, gt) - oracle_loss(sl - h * d, gt)) / (2 * h)
        ad = float(np.sum(g_sl * d))
        print(f"oracle 2D zero-gradient y: fd={fd:.10e} adjoint={ad:.10e}")
        assert abs(fd - ad) <= 1e-5 * abs(fd)


def _live_setup(lsgb_mod, prec):
    """20^3 sphere in the reference's live deformation vortex (time factor
    cos(pi t / T), T = 0.5, from t = 0.05), HCR-2 every 5 steps."""
    from lsgb import adjoint as adj
    n, steps = 20, 12
    _, G0, _, _, _, sl, sl_t = adj.workload(n, steps, reinit_interval=5)
    p = lsgb_mod.params(3, n, n, n, dx=1 / n, dy=1 / n, dz=1 / n, s_l=0.15, dt=0.5 / n / 2.2, enable_reinit=True,
                        reinit_interval=5, reinit_iterations=2)
    return adj, p, steps, G0, sl, sl_t


def _live_run(s, a, G0, sl, steps, record=False):
    s.set_fields(G0, layout="compact")
    s.set_sl_field(sl, layout="compact")
    s.set_velocity_deformation_live(0.05, 0.5)
    s.step = 0
    if record:
        a.forward(steps)
    else:
        s.advance(steps)


def test_adjoint_live_deformation_velocity_fd(cuda, lsgb_mod):
    """Live velocity (the vortex re-evaluated every step): FP64 adjoint vs
    central FD of the live FP64 forward in S_L and G0 (relative <= 1e-5)."""
    adj, p, steps, G0, sl, sl_t = _live_setup(lsgb_mod, "f64")
    with lsgb_mod.Solver(p, "f64") as s, lsgb_mod.Adjoint(s, 5) as a:
        _live_run(s, a, G0, sl_t, steps)
        a.set_target(s.get_G(layout="compact"), 1.5 * p.dx, layout="compact")

        def loss(G, f):
            _live_run(s, a, G, f, steps)
            return a.loss()

        _live_run(s, a, G0, sl, steps, record=True)
        L = a.loss(seed=True)
        a.backward()
        g_sl, g_G0, g_u = a.grad("sl"), a.grad("G0"), a.grad("u")
        assert L > 0 and np.isfinite(g_u).all() and np.abs(g_u).max() > 0
        checks = []
        for q in range(2):
            d = adj.fourier_field(sl.shape[::-1], 71 + q)
            d /= np.linalg.norm(d)
            h = 1e-6 * np.linalg.norm(sl)
            checks.append(("sl", (loss(G0, sl + h * d) - loss(G0, sl - h * d)) / (2 * h), float(np.sum(g_sl * d))))
        d = adj.fourier_field(sl.shape[::-1], 81)
        d /= np.linalg.norm(d)
        h = 1e-6 * np.linalg.norm(G0)
        checks.append(("G0", (loss(G0 + h * d, sl) - loss(G0 - h * d, sl)) / (2 * h), float(np.sum(g_G0 * d))))
    for name, fd, ad in checks:
        print(f"live {name}: fd={fd:.10e} adjoint={ad:.10e} rel={abs(fd - ad) / abs(fd):.2e}")
        assert abs(fd - ad) <= 1e-5 * abs(fd), (name, fd, ad)


def test_adjoint_live_velocity_checkpoints_and_f32(cuda, lsgb_mod):
    """Live velocity: gradients bit-identical for checkpoint intervals 1, 5
    and 50 (the vortex time is carried across segments and the recording
    and reverse streams refill their own fields), and the FP32 adjoint (whose
    forward forms the vortex inside the stage kernel) within 1e-3 relative
    L2 of the FP64 one."""
    adj, p, steps, G0, sl, sl_t = _live_setup(lsgb_mod, "f64")
    seed = np.ascontiguousarray(np.random.default_rng(5).standard_normal(G0.shape) * (np.abs(G0) < 0.2))
    out = {}
    for prec, ck in (("f64", 1), ("f64", 5), ("f64", 50), ("f32", 5)):
        with lsgb_mod.Solver(p, prec) as s, lsgb_mod.Adjoint(s, ck) as a:
            _live_run(s, a, G0, sl, steps, record=True)
            a.backward(seed, layout="compact")
            out[(prec, ck)] = (a.grad("sl"), a.grad("G0"), a.grad("w"))
    for ck in (1, 50):
        for g, g0 in zip(out[("f64", ck)], out[("f64", 5)]):
            assert np.array_equal(g, g0)
    for g32, g64 in zip(out[("f32", 5)], out[("f64", 5)]):
        rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
        print(f"live f32 vs f64 rel L2 {rel:.3e}")
        assert rel <= 1e-3


def test_gradient_independent_of_checkpoint_interval(cuda, lsgb_mod):
    adj, p, steps, G0, u, v, w, sl, sl_t = small(lsgb_mod, 3)
    res = []
    for ck in (1, 3, 50):
        prob = adj.Problem(p, G0, u, v, w, "f64", checkpoint=ck)
        try:
            prob.target(sl_t, steps)
            L, g = prob.gradient(sl, steps)
            res.append((L, g, prob.a.grad("G0"), prob.a.grad("w")))
        finally:
            prob.close()
    for r in res[1:]:
        assert r[0] == res[0][0]
        for a, b in zip(r[1:], res[0][1:]):
            assert np.array_equal(a, b)


def test_f32_adjoint_close_to_f64(cuda, lsgb_mod):
    adj, p, steps, G0, u, v, w, sl, sl_t = small(lsgb_mod, 3)
    out = {}
    for prec in ("f64", "f32"):
        prob = adj.Problem(p, G0, u, v, w, prec, checkpoint=6)
        try:
            prob.target(sl_t, steps)
            out[prec] = prob.gradient(sl, steps)[1]
        finally:
            prob.close()
    rel = np.linalg.norm(out["f32"] - out["f64"]) / np.linalg.norm(out["f64"])
    print(f"f32 vs f64 adjoint: rel L2 {rel:.3e}")
    assert rel <= 1e-3


@pytest.mark.parametrize("bc", [None, ("periodic", ZG)], ids=["periodic", "zgy"])
def test_f32_adjoint_close_to_f64_2d(cuda, lsgb_mod, bc):
    """The 2D FP32 adjoint (one cell per thread, the zero-gradient gather on
    the reference's default boundaries) against the FP64 one: relative L2
    <= 1e-3 for dL/dS_L and dL/dG0."""
    adj, p, steps, G0, u, v, w, sl, sl_t = small(lsgb_mod, 2, bc)
    out = {}
    for prec in ("f64", "f32"):
        prob = adj.Problem(p, G0, u, v, w, prec, checkpoint=6)
        try:
            prob.target(sl_t, steps)
            _, g = prob.gradient(sl, steps)
            out[prec] = (g, prob.a.grad("G0"))
        finally:
            prob.close()
    for g32, g64 in zip(out["f32"], out["f64"]):
        rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
        print(f"2D {bc}: f32 vs f64 adjoint rel L2 {rel:.3e}")
        assert rel <= 1e-3


def test_torch_rollout_gradients(cuda, lsgb_mod):
    import torch
    adj, p, steps, G0, u, v, w, sl, sl_t = small(lsgb_mod, 3)
    prob = adj.Problem(p, G0, u, v, w, "f64", checkpoint=4)
    try:
        gt = prob.target(sl_t, steps)
        L_native, g_native = prob.gradient(sl, steps)
        gG0_native = prob.a.grad("G0")
    finally:
        prob.close()
    T = lambda a, rg=False: torch.tensor(a, dtype=torch.float64, device="cuda").contiguous().requires_grad_(rg)
    tG0, tsl, tu, tv, tw = T(G0, True), T(sl, True), T(u, True), T(v), T(w)
    GT = adj.rollout(tG0, tsl, tu, tv, tw, p, steps, "f64", 4)
    L = adj.heaviside_loss(GT, T(gt), 1.5 * p.dx, p.dx ** 3)
    L.backward()
    assert abs(L.item() - L_native) <= 1e-12 * L_native
    np.testing.assert_allclose(tsl.grad.cpu().numpy(), g_native, rtol=1e-9, atol=1e-12 * np.abs(g_native).max())
    np.testing.assert_allclose(tG0.grad.cpu().numpy(), gG0_native, rtol=1e-9,
                               atol=1e-12 * np.abs(gG0_native).max())
    assert tu.grad is not None and tv.grad is None


@pytest.mark.parametrize("n,bc", [((21, 18, 15), "periodic"), ((16, 16, 9), "periodic"), ((21, 18, 15), ZG)])
def test_f32_adjoint_odd_and_ragged_grids(cuda, lsgb_mod, n, bc):
    """FP32 plane-pair coefficient pass on grids with an odd nz and ragged
    tiles, periodic and zero-gradient on every axis, against the FP64 adjoint
    (relative L2 <= 1e-3)."""
    from lsgb import adjoint as adj
    rng = np.random.default_rng(sum(n))
    shape = n[::-1]
    z, y, x = np.meshgrid(*[np.arange(q) / q for q in shape], indexing="ij")
    G0 = np.sqrt((x - 0.5) ** 2 + (y - 0.45) ** 2 + (z - 0.55) ** 2) - 0.3
    u, v, w = (0.5 * np.sin(2 * np.pi * (a + b)) for a, b in ((y, z), (z, x), (x, y)))
    sl = 0.15 + 0.05 * adj.fourier_field(n, 3)
    seed = rng.standard_normal(shape) * (np.abs(G0) < 0.2)
    p = lsgb_mod.params(3, *n, dx=1 / n[0], dy=1 / n[1], dz=1 / n[2], s_l=0.15, dt=2e-3, enable_reinit=True,
                        reinit_interval=4, reinit_iterations=2, bc_x=bc, bc_y=bc, bc_z=bc)
    out = {}
    for prec in ("f64", "f32"):
        with lsgb_mod.Solver(p, prec) as s:
            s.set_fields(*(np.ascontiguousarray(a) for a in (G0, u, v, w)), layout="compact")
            s.set_sl_field(np.ascontiguousarray(sl), layout="compact")
            with lsgb_mod.Adjoint(s, 3) as a:
                a.forward(10)
                a.backward(np.ascontiguousarray(seed), layout="compact")
                out[prec] = (a.grad("sl"), a.grad("G0"), a.grad("w"))
    for g32, g64 in zip(out["f32"], out["f64"]):
        rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
        print(f"n={n}: f32 vs f64 rel L2 {rel:.3e}")
        assert rel <= 1e-3


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("bcz", ["periodic", ZG])
def test_gradient_independent_of_z_slab(cuda, lsgb_mod, prec, bcz):
    """The stage transpose runs in z slabs (coefficients L2-resident between
    its two passes); every slab size gives the same gradients bit for bit,
    with a periodic z axis and with a clamped one (whose slab planes outside
    the grid hold no cell)."""
    from lsgb import adjoint as adj
    n = (40, 36, 30)
    shape = n[::-1]
    z, y, x = np.meshgrid(*[np.arange(q) / q for q in shape], indexing="ij")
    G0 = np.ascontiguousarray(np.sqrt((x - 0.5) ** 2 + (y - 0.45) ** 2 + (z - 0.55) ** 2) - 0.3)
    u, v, w = (np.ascontiguousarray(0.5 * np.sin(2 * np.pi * (a + b))) for a, b in ((y, z), (z, x), (x, y)))
    sl = np.ascontiguousarray(0.15 + 0.05 * adj.fourier_field(n, 4))
    seed = np.ascontiguousarray(np.random.default_rng(9).standard_normal(shape) * (np.abs(G0) < 0.15))
    p = lsgb_mod.params(3, *n, dx=1 / n[0], dy=1 / n[1], dz=1 / n[2], s_l=0.15, dt=2e-3, enable_reinit=True,
                        reinit_interval=4, reinit_iterations=2, bc_z=bcz)
    res = []
    for slab in (0, 30, 7, 1):
        with lsgb_mod.Solver(p, prec) as s:
            s.set_fields(G0, u, v, w, layout="compact")
            s.set_sl_field(sl, layout="compact")
            with lsgb_mod.Adjoint(s, 4) as a:
                a.set_slab(slab)
                a.forward(9)
                a.backward(seed, layout="compact")
                res.append((a.grad("sl"), a.grad("G0"), a.grad("u")))
    for r in res[1:]:
        for g, g0 in zip(r, res[0]):
            assert np.array_equal(g, g0)
