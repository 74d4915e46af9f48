"""Binary G dumps in the reference's .bin format (needs a GB300): byte-equal
to the files the reference's own writer (saveFieldBinary3D / saveFieldBinary,
compiled into oracle/_ref) made from the same fields, committed under
tests/golden/; the asynchronous snapshot files equal synchronous dumps."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_bytes(name):
    with open(os.path.join(GOLDEN, name), "rb") as f:
        return f.read()


def test_drop_in_dump_matches_reference_writer(cuda, lsgb_mod):
    import torch
    z = np.load(os.path.join(GOLDEN, "golden_3d_small.npz"))
    p = lsgb_mod.params(3, 12, 10, 8)
    G = torch.tensor(z["run10"], dtype=torch.float64, device="cuda")
    assert lsgb_mod.dump_f64(p, G) == golden_bytes("dump_3d_small_run10.bin")
    for tag, per in (("periodic", True), ("zerograd", False)):
        z2 = np.load(os.path.join(GOLDEN, f"golden_2d_{tag}.npz"))
        p2 = lsgb_mod.params(2, 14, 11, bc_y="periodic" if per else "zero_gradient")
        G2 = torch.tensor(z2["run9"], dtype=torch.float64, device="cuda")
        assert lsgb_mod.dump_f64(p2, G2) == golden_bytes(f"dump_2d_{tag}_run9.bin")


def test_solver_dump_matches_reference_writer(cuda, lsgb_mod):
    z = np.load(os.path.join(GOLDEN, "golden_3d_small.npz"))
    p = lsgb_mod.params(3, 12, 10, 8, s_l=float(z["s_l"]), dt=float(z["dt"]), enable_reinit=True,
                        reinit_interval=3, reinit_iterations=3)
    with lsgb_mod.Solver(p, "f64") as s:
        s.set_fields(z["G"], z["u"], z["v"], z["w"])
        s.advance(10)
        img = s.dump()
    assert img == golden_bytes("dump_3d_small_run10.bin")
    hdr, arr = lsgb_mod.read_dump(img, 3)
    assert hdr == [12, 10, 8, 3] and np.array_equal(arr, np.frombuffer(img, np.float64, offset=16).reshape(14, 16, 18))


def test_snapshots_equal_synchronous_dumps(cuda, lsgb_mod, tmp_path):
    from lsgb import synthetic as syn
    wl = syn.sphere_config(3, 40, 8, 0.2)
    wl.n = (40, 36, 44)
    G, u, v, w = syn.host_fields(wl)
    p = lsgb_mod.params(3, 40, 36, 44, dx=1 / 40, dy=1 / 36, dz=1 / 44, s_l=0.2, dt=2e-3, enable_reinit=True,
                        reinit_interval=5, reinit_iterations=2)
    with lsgb_mod.Solver(p, "f32") as a, lsgb_mod.Solver(p, "f32") as b:
        for s in (a, b):
            s.set_fields(G, u, v, w)
        want = []
        for k in range(5):  # more snapshots than slots: the third waits for the first file
            a.advance(3)
            a.snapshot(str(tmp_path / f"G_step_{k:06d}.bin"))
            b.advance(3)
            want.append(b.dump())
        a.snapshot_wait()
    for k in range(5):
        assert (tmp_path / f"G_step_{k:06d}.bin").read_bytes() == want[k]
    with lsgb_mod.Solver(p, "f32") as s:
        s.set_fields(G, u, v, w)
        s.snapshot(str(tmp_path / "no_such_dir" / "x.bin"))
        with pytest.raises(lsgb_mod.LsgbError):
            s.snapshot_wait()
