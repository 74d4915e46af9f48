"""The binary dump format, pinned on the CPU: the files the reference's own
writer produced (tests/golden/dump_*.bin, made by tests/golden/make_golden.py
through oracle/_ref) are the int32 header followed by the ghosted array with
its y ghost rows replaced by copies of the first / last interior row."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def expected(run, hdr):
    e = run.copy()
    if run.ndim == 3:
        e[:, :3, :] = run[:, 3:4, :]
        e[:, -3:, :] = run[:, -4:-3, :]
    else:
        e[:3, :] = run[3:4, :]
        e[-3:, :] = run[-4:-3, :]
    return np.asarray(hdr, dtype=np.int32).tobytes() + e.tobytes()


def test_reference_dump_layout():
    z = np.load(os.path.join(GOLDEN, "golden_3d_small.npz"))
    with open(os.path.join(GOLDEN, "dump_3d_small_run10.bin"), "rb") as f:
        assert f.read() == expected(z["run10"], [12, 10, 8, 3])
    for tag in ("periodic", "zerograd"):
        z2 = np.load(os.path.join(GOLDEN, f"golden_2d_{tag}.npz"))
        with open(os.path.join(GOLDEN, f"dump_2d_{tag}_run9.bin"), "rb") as f:
            assert f.read() == expected(z2["run9"], [14, 11, 3])


def test_read_dump_round_trip():
    import lsgb
    z = np.load(os.path.join(GOLDEN, "golden_3d_small.npz"))
    img = expected(z["run10"], [12, 10, 8, 3])
    hdr, arr = lsgb.read_dump(img, 3)
    assert hdr == [12, 10, 8, 3] and arr.shape == (14, 16, 18)
