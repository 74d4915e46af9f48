"""The CPU oracle, pinned before it is trusted (runs without a GPU).

* oracle/ls_oracle.c (the restatement) against the golden fixtures that the
  reference's own solver headers produced (tests/golden/make_golden.py);
* the restatement against the compiled reference (oracle/_ref) on fresh
  seeded cases, when the reference tree is present on this host;
* the reference's default 64^3 deformation case against the reference's
  committed log (Local_code/level-set_MPI_3D/log/simulation.log).
All comparisons are bit for bit.
"""
import json
import os

import numpy as np
import pytest

from oracle import Oracle, Problem, ref_available

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def test_port_matches_golden_3d(port):
    z = load("golden_3d_small.npz")
    pb = Problem(nx=12, ny=10, nz=8, dim=3, s_l=float(z["s_l"]), dt=float(z["dt"]), enable_reinit=True,
                 reinit_interval=3, reinit_iterations=3)
    G, u, v, w = z["G"], z["u"], z["v"], z["w"]
    assert np.array_equal(port.rk3_step(pb, G, u, v, w), z["rk3"])
    pb0 = Problem(**{**pb.__dict__, "s_l": 0.0})
    assert np.array_equal(port.rk3_step(pb0, G, u, v, w), z["rk3_sl0"])
    phi, phi0, rt, flag = port.reinit(pb, G)
    assert np.array_equal(phi, z["reinit_phi"])
    assert np.array_equal(phi0, z["reinit_phi0"])
    assert np.array_equal(rt, z["reinit_rt"])
    assert np.array_equal(flag, z["reinit_flag"])
    run = port.run(pb, 10, G, u, v, w)
    assert np.array_equal(run, z["run10"])
    assert port.volume(pb, run) == float(z["vol_run10"])
    assert port.l2(pb, run, G) == float(z["l2_run10"])


@pytest.mark.parametrize("tag,periodic", [("periodic", True), ("zerograd", False)])
def test_port_matches_golden_2d(port, tag, periodic):
    z = load(f"golden_2d_{tag}.npz")
    pb = Problem(nx=14, ny=11, dim=2, s_l=float(z["s_l"]), dt=float(z["dt"]), enable_reinit=True,
                 reinit_interval=2, reinit_iterations=2, periodic_y=periodic)
    G, u, v = z["G"], z["u"], z["v"]
    assert np.array_equal(port.rk3_step(pb, G, u, v), z["rk3"])
    phi, phi0, rt, flag = port.reinit(pb, G)
    for a, b in ((phi, "reinit_phi"), (phi0, "reinit_phi0"), (rt, "reinit_rt"), (flag, "reinit_flag")):
        assert np.array_equal(a, z[b]), b
    run = port.run(pb, 9, G, u, v)
    assert np.array_equal(run, z["run9"])
    assert port.volume(pb, run) == float(z["area_run9"])
    assert port.l2(pb, run, G) == float(z["l2_run9"])


def test_port_matches_golden_config1(port):
    from lsgb import synthetic as syn
    z = load("golden_config1_128.npz")
    G, u, v, _ = syn.host_fields(syn.config1(128))
    pb = Problem(nx=128, ny=128, dim=2, s_l=0.1, dt=float(z["dt"]), enable_reinit=True,
                 reinit_interval=10, reinit_iterations=5, periodic_y=True)
    assert port.volume(pb, G) == float(z["area0"])
    fin = port.run(pb, 400, G, u, v)
    assert np.array_equal(fin[3:-3, 3:-3], z["G_final"])
    assert port.volume(pb, fin) == float(z["area_final"])


def test_port_deformation_matches_reference_log():
    """64^3 sphere deformation, 1501 steps: the reference's committed log
    printed L2 9.158634e-04 and volume 0.014165 -> 0.014245."""
    import ctypes as C
    from oracle import build_port
    L = C.CDLL(build_port())
    l2, v0, v1, st = C.c_double(), C.c_double(), C.c_double(), C.c_int()
    L.orc3d_deformation_test(64, C.byref(l2), C.byref(v0), C.byref(v1), C.byref(st))
    gold = json.load(open(os.path.join(GOLD, "golden_scalars.json")))["deformation_64"]
    assert st.value == gold["log_steps"] == gold["steps"]
    assert f"{l2.value:.6e}" == gold["log_l2"]
    assert f"{v0.value:.6f}" == gold["log_volume_initial"]
    assert f"{v1.value:.6f}" == gold["log_volume_final"]
    assert (l2.value, v0.value, v1.value) == (gold["l2"], gold["volume_initial"], gold["volume_final"])


def zalesak_run(port, n=201):
    """The reference's 2D Zalesak loop (Local_code/level-set_MPI_2D/src/main.cpp:314-335):
    fixed dt, then the final step clipped to t_final."""
    from lsgb import synthetic as syn
    G0, u, v, dx, dt = syn.zalesak_fields(n)
    t, full = 0.0, 0
    while t < syn.ZALESAK_T_FINAL and t + dt <= syn.ZALESAK_T_FINAL:
        t += dt
        full += 1
    pb = Problem(nx=n, ny=n, dim=2, dx=dx, dy=dx, dt=dt, periodic_y=False)
    G = port.run(pb, full, G0, u, v)
    if t < syn.ZALESAK_T_FINAL:
        last = Problem(nx=n, ny=n, dim=2, dx=dx, dy=dx, dt=syn.ZALESAK_T_FINAL - t, periodic_y=False)
        G = port.run(last, 1, G, u, v)
        full += 1
    return pb, G0, G, full


def test_port_zalesak_matches_reference_log(port):
    """The reference's 2D known answer: Zalesak's disk rotated once on 201^2
    (log Local_code/level-set_MPI_2D/log/201x201.log).  The restated initial
    field and the port's final field equal the compiled reference's (SHA-256
    of the interiors); the scalars equal its values and the log's printed
    L2, final area and step count."""
    import hashlib
    gold = json.load(open(os.path.join(GOLD, "golden_zalesak_201.json")))
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a[3:-3, 3:-3]).tobytes()).hexdigest()
    pb, G0, G, steps = zalesak_run(port)
    assert sha(G0) == gold["G0_sha256"]
    assert sha(G) == gold["G_final_sha256"]
    assert steps == gold["steps"] == gold["log"]["steps"]
    l2, a0, a1 = port.l2(pb, G, G0), port.volume(pb, G0), port.volume(pb, G)
    assert (l2, a0, a1) == (gold["l2"], gold["area_initial"], gold["area_final"])
    assert f"{l2:.6e}" == gold["log"]["l2"] and f"{a1:.6f}" == gold["log"]["area_final"]


needs_ref = pytest.mark.skipif(not ref_available(), reason="oracle/_ref not built (no reference tree)")


@needs_ref
@pytest.mark.parametrize("dim,periodic,s_l,nx,ny,nz", [
    (3, True, 0.2, 9, 7, 6), (3, True, 0.0, 5, 4, 3), (3, True, 0.3, 16, 3, 5),
    (2, True, 0.05, 3, 3, 1), (2, False, 0.2, 17, 6, 1), (2, False, 0.0, 8, 21, 1),
])
def test_port_matches_reference(port, dim, periodic, s_l, nx, ny, nz):
    ref = Oracle("ref")
    rng = np.random.default_rng(nx * 100 + ny)
    pb = Problem(nx=nx, ny=ny, nz=nz, dim=dim, s_l=s_l, dt=1.5e-3, enable_reinit=True,
                 reinit_interval=2, reinit_iterations=3, periodic_y=periodic)
    G = rng.standard_normal(pb.shape) * 0.1 + 0.02
    vel = [rng.standard_normal(pb.shape) for _ in range(dim)]
    args = (G, *vel)
    assert np.array_equal(port.rk3_step(pb, *args), ref.rk3_step(pb, *args))
    assert np.array_equal(port.rhs(pb, *args), ref.rhs(pb, *args))
    assert np.array_equal(port.apply_bc(pb, G), ref.apply_bc(pb, G))
    for a, b in zip(port.reinit(pb, G), ref.reinit(pb, G)):
        assert np.array_equal(a, b)
    ra, rb = port.run(pb, 7, *args), ref.run(pb, 7, *args)
    assert np.array_equal(ra, rb)
    assert port.volume(pb, ra) == ref.volume(pb, rb)
    assert port.l2(pb, ra, G) == ref.l2(pb, rb, G)


def test_port_segmented_run_equals_single_run(port):
    """Step counter offset keeps the reinit cadence across segments."""
    rng = np.random.default_rng(7)
    pb = Problem(nx=8, ny=9, nz=7, dim=3, s_l=0.1, dt=1e-3, enable_reinit=True, reinit_interval=3,
                 reinit_iterations=2)
    G = rng.standard_normal(pb.shape) * 0.1
    vel = [rng.standard_normal(pb.shape) for _ in range(3)]
    one = port.run(pb, 8, G, *vel)
    a = port.run(pb, 5, G, *vel)
    two = port.run(pb, 3, a, *vel, step0=5)
    assert np.array_equal(one, two)
