"""FP64 parity of the CUDA path against the oracle (needs a GB300).

Bit-for-bit (np.array_equal) against:
* the golden fixtures the reference's own solver produced (tests/golden/),
* the C restatement (oracle/ls_oracle.c) on fresh seeded inputs, including
  ragged sizes, the 3-cell minimum, zero-gradient Y and a per-cell S_L field,
and the reference's committed 64^3 deformation log.  Everything goes through
the C ABI (lsgb_*), drop-in entry points and solver handle alike.
"""
import json
import os

import numpy as np
import pytest

from oracle import Problem

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def lsgb_params(lsgb, pb: Problem):
    return lsgb.params(pb.dim, pb.nx, pb.ny, pb.nz, dx=pb.dx, dy=pb.dy, dz=pb.dz, dt=pb.dt,
                       s_l=pb.s_l, epsilon=pb.epsilon, enable_reinit=pb.enable_reinit,
                       reinit_interval=pb.reinit_interval, reinit_iterations=pb.reinit_iterations,
                       reinit_dtau=pb.reinit_dtau, reinit_beta=pb.reinit_beta,
                       bc_y=0 if pb.periodic_y else 1)


def dropin_step(lsgb, p, G, u, v, w=None, sl=None):
    import torch
    Gd = dev(G)
    out = [torch.zeros_like(Gd) for _ in range(3)]
    lsgb.rk3_step_f64(p, Gd, out[0], out[1], out[2], dev(u), dev(v), None if w is None else dev(w),
                      None if sl is None else dev(sl))
    return host(out[0])


def dropin_reinit(lsgb, p, G):
    import torch
    phi = dev(G)
    tmp = torch.zeros_like(phi)
    phi0 = torch.zeros_like(phi)
    rt = torch.zeros_like(phi)
    flag = torch.zeros(phi.shape, dtype=torch.int32, device=phi.device)
    res, _ = lsgb.reinit_f64(p, phi, tmp, phi0, rt, flag)
    return host(res), host(phi0), host(rt), host(flag)


def solver_run(lsgb, p, n, G, u, v, w=None, sl=None, precision="f64", tile=0):
    with lsgb.Solver(p, precision) as s:
        s.set_tile(tile)
        s.set_fields(G, u, v, w)
        if sl is not None:
            s.set_sl_field(sl)
        s.advance(n)
        return s.get_G(), s.volume()


# -- golden fixtures (the reference's own output) ---------------------------
def test_golden_3d(cuda, lsgb_mod):
    z = load("golden_3d_small.npz")
    pb = Problem(nx=12, ny=10, nz=8, dim=3, s_l=float(z["s_l"]), dt=float(z["dt"]), enable_reinit=True,
                 reinit_interval=3, reinit_iterations=3)
    p = lsgb_params(lsgb_mod, pb)
    G, u, v, w = z["G"], z["u"], z["v"], z["w"]
    assert np.array_equal(dropin_step(lsgb_mod, p, G, u, v, w), z["rk3"])
    p0 = lsgb_params(lsgb_mod, Problem(**{**pb.__dict__, "s_l": 0.0}))
    assert np.array_equal(dropin_step(lsgb_mod, p0, G, u, v, w), z["rk3_sl0"])
    phi, phi0, rt, flag = dropin_reinit(lsgb_mod, p, G)
    assert np.array_equal(phi, z["reinit_phi"])
    assert np.array_equal(phi0, z["reinit_phi0"])
    assert np.array_equal(rt, z["reinit_rt"])
    assert np.array_equal(flag, z["reinit_flag"])
    out, (vol, cnt) = solver_run(lsgb_mod, p, 10, G, u, v, w)
    assert np.array_equal(out, z["run10"])
    assert cnt == int((z["run10"][3:-3, 3:-3, 3:-3] < 0).sum())
    assert vol == pytest.approx(float(z["vol_run10"]), rel=1e-12)


@pytest.mark.parametrize("tag,periodic", [("periodic", True), ("zerograd", False)])
def test_golden_2d(cuda, lsgb_mod, tag, periodic):
    z = load(f"golden_2d_{tag}.npz")
    pb = Problem(nx=14, ny=11, dim=2, s_l=float(z["s_l"]), dt=float(z["dt"]), enable_reinit=True,
                 reinit_interval=2, reinit_iterations=2, periodic_y=periodic)
    p = lsgb_params(lsgb_mod, pb)
    G, u, v = z["G"], z["u"], z["v"]
    assert np.array_equal(dropin_step(lsgb_mod, p, G, u, v), z["rk3"])
    phi, phi0, rt, flag = dropin_reinit(lsgb_mod, p, G)
    for a, b in ((phi, "reinit_phi"), (phi0, "reinit_phi0"), (rt, "reinit_rt"), (flag, "reinit_flag")):
        assert np.array_equal(a, z[b]), b
    out, (area, cnt) = solver_run(lsgb_mod, p, 9, G, u, v)
    assert np.array_equal(out, z["run9"])
    assert area == pytest.approx(float(z["area_run9"]), rel=1e-12)


def test_golden_config1(cuda, lsgb_mod):
    """2D 128^2 circle, u = (1, 0), S_L = 0.1, CFL 0.5, 400 steps, HCR-2 every 10 x 5."""
    from lsgb import synthetic as syn
    z = load("golden_config1_128.npz")
    G, u, v, _ = syn.host_fields(syn.config1(128))
    pb = Problem(nx=128, ny=128, dim=2, s_l=0.1, dt=float(z["dt"]), enable_reinit=True,
                 reinit_interval=10, reinit_iterations=5, periodic_y=True)
    out, (area, _) = solver_run(lsgb_mod, lsgb_params(lsgb_mod, pb), 400, G, u, v)
    assert np.array_equal(out[3:-3, 3:-3], z["G_final"])
    assert area == pytest.approx(float(z["area_final"]), rel=1e-12)


def test_deformation_64_matches_reference_log(cuda, lsgb_mod, port):
    """The reference's default case: 64^3 sphere in the deformation vortex,
    dx = 1/63, dt = 1e-3 with the final-step clip, 1501 steps, velocity
    recomputed on the device every step (Local_code/level-set_MPI_3D/src/main.cpp:291-334)."""
    import ctypes as C
    from oracle import build_port
    L = C.CDLL(build_port())
    n, T = 64, 1.5
    pb = Problem(nx=n, ny=n, nz=n, dim=3, dx=1 / 63, dy=1 / 63, dz=1 / 63, dt=1e-3)
    G0 = np.zeros(pb.shape)
    L.orc3d_sphere(C.byref(pb.c()), C.c_double(0.35), C.c_double(0.35), C.c_double(0.35),
                   C.c_double(0.15), G0.ctypes.data_as(C.POINTER(C.c_double)))
    G0 = port.apply_bc(pb, G0)
    p = lsgb_params(lsgb_mod, pb)
    with lsgb_mod.Solver(p, "f64") as s:
        s.set_fields(G=G0)
        v0, _ = s.volume()
        t, dt, steps = 0.0, 1e-3, 0
        while t < T and steps < int(T / 1e-3) + 100:
            if t + dt > T:
                dt = T - t
                s.set_dt(dt)
            s.set_velocity_deformation(t, T)
            s.advance(1)
            t += dt
            steps += 1
        v1, _ = s.volume()
        l2 = s.l2_error(G0)
    gold = json.load(open(os.path.join(GOLD, "golden_scalars.json")))["deformation_64"]
    assert steps == gold["log_steps"]
    assert f"{l2:.6e}" == gold["log_l2"]
    assert f"{v0:.6f}" == gold["log_volume_initial"]
    assert f"{v1:.6f}" == gold["log_volume_final"]
    assert l2 == pytest.approx(gold["l2"], rel=1e-9)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_deformation_64_live_velocity(cuda, lsgb_mod, port, prec):
    """The same case with the velocity in live mode (the handle recomputes the
    vortex every step; inside the stage kernel for FP32 on this grid).  FP64
    reproduces the log and the port's L2 as the explicit loop does; FP32 stays
    within 1e-3 of the log's L2 and within 5 cells of its final volume."""
    import ctypes as C
    from oracle import build_port
    L = C.CDLL(build_port())
    n, T, dt = 64, 1.5, 1e-3
    pb = Problem(nx=n, ny=n, nz=n, dim=3, dx=1 / 63, dy=1 / 63, dz=1 / 63, dt=dt)
    G0 = np.zeros(pb.shape)
    L.orc3d_sphere(C.byref(pb.c()), C.c_double(0.35), C.c_double(0.35), C.c_double(0.35),
                   C.c_double(0.15), G0.ctypes.data_as(C.POINTER(C.c_double)))
    G0 = port.apply_bc(pb, G0)
    with lsgb_mod.Solver(lsgb_params(lsgb_mod, pb), prec) as s:
        s.set_fields(G=G0)
        v0, _ = s.volume()
        s.set_velocity_deformation_live(0.0, T)
        s.advance(1400)
        steps = 1400
        t = s.time()
        while t < T and steps < int(T / 1e-3) + 100:  # the reference's loop with its final-step clip
            if t + dt > T:
                dt = T - t
                s.set_dt(dt)
            s.advance(1)
            t = s.time()
            steps += 1
        v1, _ = s.volume()
        l2 = s.l2_error(G0)
    gold = json.load(open(os.path.join(GOLD, "golden_scalars.json")))["deformation_64"]
    assert steps == gold["log_steps"]
    if prec == "f64":
        assert f"{l2:.6e}" == gold["log_l2"]
        assert f"{v0:.6f}" == gold["log_volume_initial"] and f"{v1:.6f}" == gold["log_volume_final"]
        assert l2 == pytest.approx(gold["l2"], rel=1e-9)
    else:
        assert l2 == pytest.approx(gold["l2"], rel=1e-3)
        assert abs(v1 - gold["volume_final"]) <= 5 * (1 / 63) ** 3


def zalesak_gpu(lsgb, n):
    """The reference's Zalesak loop on the FP64 handle: returns the final
    ghosted G, its L2 error against G0, the final area and cell count, the
    initial area and the step count."""
    from lsgb import synthetic as syn
    G0, u, v, dx, dt = syn.zalesak_fields(n)
    p = lsgb.params(2, n, n, 1, dx=dx, dy=dx, dt=dt, s_l=0.0, enable_reinit=False, bc_y=1)
    with lsgb.Solver(p, "f64") as s:
        s.set_fields(G0, u, v)
        a0, _ = s.volume()
        t, steps = 0.0, 0
        while t < syn.ZALESAK_T_FINAL:
            if t + dt > syn.ZALESAK_T_FINAL:
                dt = syn.ZALESAK_T_FINAL - t
                s.set_dt(dt)
            s.advance(1)
            t += dt
            steps += 1
        G = s.get_G()
        l2 = s.l2_error(G0)
        area, count = s.volume()
    return G, l2, area, count, a0, steps


# printed values of the reference's logs (Local_code/level-set_MPI_2D/log/<n>x<n>.log)
ZALESAK_LOGS = {401: ("8.373019e-02", "0.058081", 12567), 801: ("8.250949e-02", "0.058311", 25133)}


@pytest.mark.parametrize("n", [401, 801])
def test_zalesak_larger_grids_match_reference_logs(cuda, lsgb_mod, n):
    """The same known answer on the 401^2 and 801^2 logs: the printed L2,
    final area and step count."""
    _, l2, area, _, a0, steps = zalesak_gpu(lsgb_mod, n)
    print(f"n={n}: l2={l2:.6e} area0={a0:.6f} area={area:.6f} steps={steps}")
    log_l2, log_area, log_steps = ZALESAK_LOGS[n]
    assert steps == log_steps
    assert f"{l2:.6e}" == log_l2 and f"{area:.6f}" == log_area


def test_zalesak_201_matches_reference(cuda, lsgb_mod):
    """The reference's 2D known answer (Zalesak's disk rotated once on 201^2,
    periodic X, zero-gradient Y, 6284 steps with the final-step clip;
    Local_code/level-set_MPI_2D/log/201x201.log) through the FP64 handle: the
    final field equals the compiled reference's bit for bit (SHA-256 of the
    interior) and the printed L2 and final area match the log."""
    import hashlib
    gold = json.load(open(os.path.join(GOLD, "golden_zalesak_201.json")))
    G, l2, area, count, _, steps = zalesak_gpu(lsgb_mod, gold["n"])
    sha = hashlib.sha256(np.ascontiguousarray(G[3:-3, 3:-3]).tobytes()).hexdigest()
    assert steps == gold["steps"]
    assert sha == gold["G_final_sha256"]
    assert count == gold["negative_cells_final"]
    assert f"{l2:.6e}" == gold["log"]["l2"] and f"{area:.6f}" == gold["log"]["area_final"]
    assert l2 == pytest.approx(gold["l2"], rel=1e-12)


# -- fresh seeded cases against the C restatement -----------------------------
CASES = [
    (3, True, 0.2, 13, 11, 9), (3, True, 0.0, 3, 3, 3), (3, True, 0.25, 33, 5, 17),
    (3, True, 0.1, 40, 36, 6), (2, True, 0.1, 3, 3, 1), (2, False, 0.2, 37, 9, 1),
    (2, True, 0.0, 64, 31, 1), (2, False, 0.3, 5, 70, 1),
]


def seeded(pb: Problem, seed: int):
    rng = np.random.default_rng(seed)
    G = rng.standard_normal(pb.shape) * 0.1 + 0.01
    vel = [rng.standard_normal(pb.shape) for _ in range(pb.dim)]
    sl = np.abs(rng.standard_normal(pb.shape)) * 0.2
    sl[rng.random(pb.shape) < 0.2] = 0.0  # exercise the s_l > epsilon gate per cell
    return G, vel, sl


@pytest.mark.parametrize("dim,periodic,s_l,nx,ny,nz", CASES)
def test_against_port(cuda, lsgb_mod, port, dim, periodic, s_l, nx, ny, nz):
    pb = Problem(nx=nx, ny=ny, nz=nz, dim=dim, s_l=s_l, dt=1.3e-3, enable_reinit=True,
                 reinit_interval=2, reinit_iterations=3, periodic_y=periodic)
    p = lsgb_params(lsgb_mod, pb)
    G, vel, sl = seeded(pb, nx * 1000 + ny * 10 + nz)
    w = vel[2] if dim == 3 else None
    assert np.array_equal(dropin_step(lsgb_mod, p, G, vel[0], vel[1], w), port.rk3_step(pb, G, *vel))
    assert np.array_equal(dropin_step(lsgb_mod, p, G, vel[0], vel[1], w, sl=sl),
                          port.rk3_step(pb, G, *vel, sl=sl))
    for a, b in zip(dropin_reinit(lsgb_mod, p, G), port.reinit(pb, G)):
        assert np.array_equal(a, b)
    ref = port.run(pb, 7, G, *vel)
    out, (vol, cnt) = solver_run(lsgb_mod, p, 7, G, vel[0], vel[1], w)
    assert np.array_equal(out, ref)
    interior = ref[(slice(3, -3),) * dim]
    assert cnt == int((interior < 0).sum())
    out, _ = solver_run(lsgb_mod, p, 5, G, vel[0], vel[1], w, sl=sl)
    assert np.array_equal(out, port.run(pb, 5, G, *vel, sl=sl))


@pytest.mark.parametrize("dim,periodic,s_l,nx,ny,nz", CASES)
@pytest.mark.parametrize("tile", [1, 2])
def test_fp64_kernel_forms_match_port(cuda, lsgb_mod, port, dim, periodic, s_l, nx, ny, nz, tile):
    """Both FP64 stage kernels -- one thread per cell (tile 1) and the
    face-shared tiles (tile 2, each face value computed once) -- on ragged
    grids, uniform and per-cell S_L, periodic and zero-gradient Y."""
    pb = Problem(nx=nx, ny=ny, nz=nz, dim=dim, s_l=s_l, dt=1.3e-3, enable_reinit=True,
                 reinit_interval=2, reinit_iterations=3, periodic_y=periodic)
    p = lsgb_params(lsgb_mod, pb)
    G, vel, sl = seeded(pb, nx * 1000 + ny * 10 + nz + 7)
    w = vel[2] if dim == 3 else None
    out, _ = solver_run(lsgb_mod, p, 5, G, vel[0], vel[1], w, tile=tile)
    assert np.array_equal(out, port.run(pb, 5, G, *vel))
    out, _ = solver_run(lsgb_mod, p, 4, G, vel[0], vel[1], w, sl=sl, tile=tile)
    assert np.array_equal(out, port.run(pb, 4, G, *vel, sl=sl))


@pytest.mark.parametrize("dim,periodic,n", [(3, True, (97, 45, 41)), (2, True, (650, 261, 1)),
                                            (2, False, (650, 261, 1))])
def test_dropin_face_shared_tiles_match_port(cuda, lsgb_mod, port, dim, periodic, n):
    """The drop-in step on ghosted arrays at sizes where the face-shared FP64
    kernel is the default (every SM gets two tiles), ragged tiles at the edges."""
    pb = Problem(nx=n[0], ny=n[1], nz=n[2], dim=dim, s_l=0.15, dt=1e-3, periodic_y=periodic)
    p = lsgb_params(lsgb_mod, pb)
    G, vel, sl = seeded(pb, 91)
    G, vel = port.apply_bc(pb, G), [port.apply_bc(pb, a) for a in vel]
    w = vel[2] if dim == 3 else None
    assert np.array_equal(dropin_step(lsgb_mod, p, G, vel[0], vel[1], w), port.rk3_step(pb, G, *vel))
    assert np.array_equal(dropin_step(lsgb_mod, p, G, vel[0], vel[1], w, sl=sl), port.rk3_step(pb, G, *vel, sl=sl))


def test_reductions_match_port(cuda, lsgb_mod, port):
    pb = Problem(nx=21, ny=17, nz=11, dim=3)
    p = lsgb_params(lsgb_mod, pb)
    G, vel, _ = seeded(pb, 5)
    G2 = G + 0.01
    assert lsgb_mod.l2_error_f64(p, dev(G), dev(G2)) == pytest.approx(port.l2(pb, G, G2), rel=1e-13)
    assert lsgb_mod.max_speed_f64(p, *[dev(a) for a in vel]) == port.max_speed(pb, *vel)
    vol, cnt = lsgb_mod.volume_f64(p, dev(G))
    assert cnt == int((G[3:-3, 3:-3, 3:-3] < 0).sum())
    assert vol == pytest.approx(port.volume(pb, G), rel=1e-12)


def test_apply_bc_matches_port(cuda, lsgb_mod, port):
    for dim, per in ((3, True), (2, True), (2, False)):
        pb = Problem(nx=9, ny=8, nz=7, dim=dim, periodic_y=per)
        G, _, _ = seeded(pb, 11)
        Gd = dev(G)
        lsgb_mod.apply_bc_f64(lsgb_params(lsgb_mod, pb), Gd)
        assert np.array_equal(host(Gd), port.apply_bc(pb, G))


def test_segmented_advance_keeps_reinit_cadence(cuda, lsgb_mod, port):
    pb = Problem(nx=10, ny=9, nz=8, dim=3, s_l=0.1, dt=1e-3, enable_reinit=True, reinit_interval=3,
                 reinit_iterations=2)
    G, vel, _ = seeded(pb, 3)
    with lsgb_mod.Solver(lsgb_params(lsgb_mod, pb), "f64") as s:
        s.set_fields(G, *vel)
        s.advance(5)
        s.advance(3)
        assert s.step == 8
        out = s.get_G()
    assert np.array_equal(out, port.run(pb, 8, G, *vel))
