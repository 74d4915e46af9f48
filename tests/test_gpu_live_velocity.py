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


def test_live_rejected_by_batch_accepted_by_adjoint(cuda, lsgb_mod):
    n = (32, 32, 32)
    with make(lsgb_mod, "f32", n, 0) as s:
        s.set_velocity_deformation_live(0.0, T)
        with lsgb_mod.Adjoint(s, 4) as a:
            a.forward(6)
            a.backward(np.ones((32, 32, 32)), layout="compact")
            assert np.isfinite(a.grad("sl")).all()
        assert abs(s.time() - 6 * s.params().dt) < 1e-12  # the forward advanced the vortex time
    h = 1.0 / 31
    with lsgb_mod.Batch("f32", lanes=2) as b:
        p = lsgb_mod.params(3, *n, dx=h, dy=h, dz=h, dt=2e-3)
        s = b.add(p)
        G = sphere(n, (h, h, h))
        zero = np.zeros_like(G)
        s.set_fields(G, zero, zero, zero, layout="compact")
        s.set_velocity_deformation_live(0.0, T)
        with pytest.raises(lsgb_mod.LsgbError) as e:
            b.advance(1)
        assert e.value.code == lsgb_mod.ERR_UNSUPPORTED
        s.set_velocity_deformation(0.0, T)  # arrays again: the batch runs
        b.advance(1)
        b.sync()
