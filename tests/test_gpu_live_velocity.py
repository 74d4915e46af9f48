"""Live deformation velocity (needs a GB300).

lsgb_solver_set_velocity_deformation_live runs the reference's time loop
(Local_code/level-set_MPI_3D/src/main.cpp:291-316: velocity at current_time,
RK3 step, reinit, current_time += dt) inside one advance.  On FP32 3D grids
with nx % 4 == 0 the vortex is evaluated inside the stage kernel; elsewhere
u, v, w are refilled before each step.  Both must equal the explicit
per-step loop (set_velocity_deformation + advance(1)) bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

T = 1.5


def sphere(n, h):
    z, y, x = np.meshgrid(*[np.arange(q) * hq for q, hq in zip(n[::-1], h[::-1])], indexing="ij")
    return np.ascontiguousarray(np.sqrt((x - 0.35) ** 2 + (y - 0.35) ** 2 + (z - 0.35) ** 2) - 0.15)


def make(lsgb, prec, n, bc):
    h = tuple(1.0 / (q - 1) for q in n)
    p = lsgb.params(3, *n, dx=h[0], dy=h[1], dz=h[2], dt=2e-3, s_l=0.05, enable_reinit=True,
                    reinit_interval=3, reinit_iterations=2, bc_x=bc, bc_y=bc, bc_z=bc)
    s = lsgb.Solver(p, prec)
    G = sphere(n, h)
    zero = np.zeros_like(G)
    s.set_fields(G, zero, zero, zero, layout="compact")
    return s


@pytest.mark.parametrize("prec,n,bc", [("f32", (48, 40, 36), 0),   # vortex inside the stage kernel
                                       ("f32", (44, 24, 21), 1),   # same, zero-gradient, odd nz
                                       ("f32", (37, 21, 30), 0),   # nx % 4 != 0: refilled arrays
                                       ("f64", (30, 26, 22), 0)])
def test_live_equals_per_step_loop(cuda, lsgb_mod, prec, n, bc):
    steps, t0 = 8, 0.25
    with make(lsgb_mod, prec, n, bc) as s:
        s.set_velocity_deformation_live(t0, T)
        s.advance(steps)
        live = s.get_G(layout="compact")
        t_live = s.time()
        u_live = s.get_field("u", layout="compact")
    with make(lsgb_mod, prec, n, bc) as s:
        t = t0
        for _ in range(steps):
            s.set_velocity_deformation(t, T)
            s.advance(1)
            t += 2e-3
        loop = s.get_G(layout="compact")
        s.set_velocity_deformation(t, T)
        u_loop = s.get_field("u", layout="compact")
    assert t_live == t
    assert np.array_equal(live, loop)
    assert np.array_equal(u_live, u_loop)
    assert float(np.abs(live - sphere(n, tuple(1.0 / (q - 1) for q in n))).max()) > 1e-4  # the front moved


def test_live_accepted_by_adjoint(cuda, lsgb_mod):
    n = (32, 32, 32)
    with make(lsgb_mod, "f32", n, 0) as s:
        s.set_velocity_deformation_live(0.0, T)
        with lsgb_mod.Adjoint(s, 4) as a:
            a.forward(6)
            a.backward(np.ones((32, 32, 32)), layout="compact")
            assert np.isfinite(a.grad("sl")).all()
        assert abs(s.time() - 6 * s.params().dt) < 1e-12  # the forward advanced the vortex time


# (grid, live, zero-gradient): FP32 grids with nx % 4 == 0 form the vortex
# inside the stage kernel when run alone; in a batch every live instance
# refills u, v, w from the batch's per-step time table
BATCH_CASES = [((32, 28, 24), True, 0), ((37, 21, 30), True, 1), ((24, 24, 20), False, 0), ((36, 32, 18), True, 0)]


def _batch_instance(lsgb, s, n, live, t0):
    h = tuple(1.0 / (q - 1) for q in n)
    G = sphere(n, h)
    if live:
        s.set_fields(G, layout="compact")
        s.set_velocity_deformation_live(t0, T)
    else:
        s.set_fields(G, *(0.3 * np.ones_like(G) for _ in range(3)), layout="compact")


def _params(lsgb, n, bc):
    h = tuple(1.0 / (q - 1) for q in n)
    return lsgb.params(3, *n, dx=h[0], dy=h[1], dz=h[2], dt=2e-3, s_l=0.05, enable_reinit=True,
                       reinit_interval=3, reinit_iterations=2, bc_x=bc, bc_y=bc, bc_z=bc)


@pytest.mark.parametrize("prec,mode", [("f32", "grouped"), ("f32", "lanes"), ("f64", "lanes")])
def test_batch_live_equals_solver(cuda, lsgb_mod, prec, mode):
    """Batched live instances (the vortex time of every step read from a
    device table that replayed graphs index by a device-side cursor) equal
    the same instances advanced alone in live mode, bit for bit, beside a
    fixed-velocity instance; two advance calls (7 + 11 steps) cover the
    direct head, the graph replays, the tail and the table's reuse."""
    chunks = (7, 11)
    alone = []
    for q, (n, live, bc) in enumerate(BATCH_CASES):
        with lsgb_mod.Solver(_params(lsgb_mod, n, bc), prec) as s:
            _batch_instance(lsgb_mod, s, n, live, 0.1 * q)
            for c in chunks:
                s.advance(c)
            alone.append((s.get_G(layout="compact"), s.time()))
    with lsgb_mod.Batch(prec, lanes=3) as b:
        b.set_mode(mode)
        inst = []
        for q, (n, live, bc) in enumerate(BATCH_CASES):
            x = b.add(_params(lsgb_mod, n, bc))
            _batch_instance(lsgb_mod, x, n, live, 0.1 * q)
            inst.append(x)
        for c in chunks:
            b.advance(c)
        b.sync()
        assert b.mode == mode
        for x, (G, t), (n, live, bc) in zip(inst, alone, BATCH_CASES):
            assert np.array_equal(x.get_G(layout="compact"), G), (n, live)
            if live:
                assert x.time() == t
