"""The sample-surface oracle (oracle/ls_oracle_sample.c) against the
reference's own compiled sources (oracle/_ref/libref_sample.so, when the
reference tree is present) and the committed golden fixtures made from them.
CPU only."""
import os

import numpy as np
import pytest

from oracle import SampleOracle
from oracle.oracle import REF_DIR

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(tag):
    return np.load(os.path.join(GOLDEN, f"golden_sample_{tag}.npz"))


@pytest.fixture(scope="module")
def sport():
    return SampleOracle("port")


@pytest.mark.parametrize("tag", ["24x20", "3x3"])
def test_port_matches_golden(sport, tag):
    g = golden(tag)
    G, G0, u, v = g["G"], g["G0"], g["u"], g["v"]
    dx, dy, dt, sl = float(g["dx"]), float(g["dy"]), float(g["dt"]), float(g["S_L"])
    assert np.array_equal(sport.rhs(G, u, v, dx, dy, sl), g["rhs"])
    assert np.array_equal(sport.rk3_step(G, u, v, dx, dy, dt, sl, G0), g["rk3"])
    assert np.array_equal(sport.apply_periodic(G), g["periodic"])
    assert np.array_equal(sport.apply_anchored_bc(G, G0), g["anchored"])
    assert np.array_equal(sport.reinitialize(G, G0, dx, dy, 10), g["reinit10"])
    assert np.array_equal(sport.first_order_upwind(G, u, v, dx, dy, dt, sl), g["fou"])
    out, t = sport.run(G, G0, 25, dx, dy, dt, sl, 0.0, 0.8, 0.05, 0.05, 0)
    assert np.array_equal(out, g["run25_f0"]) and t == float(g["t25_f0"])
    out, t = sport.run(G, G0, 25, dx, dy, dt, sl, 0.0, 0.8, 0.05, 0.05, 50)
    assert np.array_equal(out, g["run25_f50"]) and t == float(g["t25_f50"])


@pytest.mark.skipif(not os.path.exists(os.path.join(REF_DIR, "libref_sample.so")),
                    reason="reference tree absent: oracle/_ref not built")
@pytest.mark.parametrize("nx,ny", [(40, 36), (3, 3), (17, 29), (5, 4)])
def test_port_matches_reference(sport, nx, ny):
    from lsgb import sample as smp
    ref = SampleOracle("ref")
    rng = np.random.default_rng(nx * 100 + ny)
    G0 = smp.bunsen(nx, ny)
    dx, dy = smp.spacing(nx, ny)
    G = np.ascontiguousarray(G0 + 1e-4 * rng.standard_normal(G0.shape))
    u = np.ascontiguousarray(0.2 * rng.standard_normal(G0.shape))
    v = np.ascontiguousarray(0.8 + 0.2 * rng.standard_normal(G0.shape))
    for name, args in [("rhs", (G, u, v, dx, dy, 0.4)), ("rk3_step", (G, u, v, dx, dy, 2e-4, 0.4, G0)),
                       ("apply_periodic", (G,)), ("apply_anchored_bc", (G, G0)),
                       ("reinitialize", (G, G0, dx, dy, 7)),
                       ("first_order_upwind", (G, u, v, dx, dy, 2e-4, 0.4))]:
        assert np.array_equal(getattr(sport, name)(*args), getattr(ref, name)(*args)), name
    a, ta = sport.run(G, G0, 12, dx, dy, 2e-4, 0.4, 0.0, 0.8, 0.05, 0.05, 120)
    b, tb = ref.run(G, G0, 12, dx, dy, 2e-4, 0.4, 0.0, 0.8, 0.05, 0.05, 120)
    assert np.array_equal(a, b) and ta == tb
