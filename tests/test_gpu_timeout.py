"""The bounded-wait failure path of the TMA-fed stage kernel (needs a GB300).

With the test hook on, the kernel issues no bulk copies: every CTA's mbarrier
wait runs into its limit (about a second of SM clock), the kernel sets the
handle's device error flag and returns.  The next synchronising call must
report LSGB_ERR_CUDA with the wait message, the flag must be cleared by that
report, and the same handle must then step normally and give the same field
as a fresh handle (the context stays usable).  No fault, trap or unbounded
wait is involved: the wait ends by its own limit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def case(lsgb):
    n = 32  # nx % 4 == 0: the bulk-tensor (TMA) form; one 32 x 16 x 16 chunk per CTA
    z, y, x = np.meshgrid(*[np.arange(n) / n] * 3, indexing="ij")
    G = np.ascontiguousarray(np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2) - 0.3)
    u = np.ascontiguousarray(np.sin(2 * np.pi * y))
    v = np.ascontiguousarray(np.sin(2 * np.pi * z))
    w = np.ascontiguousarray(np.sin(2 * np.pi * x))
    p = lsgb.params(3, n, n, n, s_l=0.2, dt=5e-3, enable_reinit=False)
    return p, (G, u, v, w)


def test_wait_limit_reports_and_recovers(cuda, lsgb_mod):
    import time
    p, f = case(lsgb_mod)
    with lsgb_mod.Solver(p, "f32") as s:
        s.set_fields(*f, layout="compact")
        s.debug_drop_copies(True)
        t0 = time.perf_counter()
        s.advance(1)  # three stage launches, each CTA gives up after its limit
        with pytest.raises(lsgb_mod.LsgbError) as e:
            s.get_G(layout="compact")
        waited = time.perf_counter() - t0
        assert e.value.code == lsgb_mod.ERR_CUDA and "bounded in-kernel wait" in str(e.value)
        assert 0.5 < waited < 60.0
        # the report cleared the flag; the handle steps normally again
        s.debug_drop_copies(False)
        s.set_fields(*f, layout="compact")
        s.step = 0
        s.advance(2)
        got = s.get_G(layout="compact")
    with lsgb_mod.Solver(p, "f32") as s:
        s.set_fields(*f, layout="compact")
        s.advance(2)
        ref = s.get_G(layout="compact")
    assert np.array_equal(got, ref)
