"""The C ABI without a GPU: the library loads, exports every declared entry
point, and its host-side logic (parameter defaults and checks, the CFL
formula, error reporting) behaves like the reference's."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT, gpu_available


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            src = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"LSGB_API\s+[\w\s\*]+?\b(lsgb_\w+)\s*\(", src))
    return sorted(names)


def test_every_declared_symbol_is_exported(lsgb_mod):
    names = declared_symbols()
    assert len(names) >= 30
    lib = lsgb_mod.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_params_default_mirrors_reference(lsgb_mod):
    p = lsgb_mod.params(3, 64, 32, 16)
    # Local_code/level-set_MPI_3D/include/config.h:88-107
    assert (p.nghost, p.reinit_interval, p.reinit_iterations) == (3, 10, 2)
    assert p.reinit_beta == 0.5 and p.epsilon == 1e-10
    assert p.reinit_dtau == 0.25 * min(1 / 64, 1 / 32, 1 / 16)
    assert p.dx == 1 / 64 and p.dy == 1 / 32 and p.dz == 1 / 16
    lsgb_mod.check_params(p)


@pytest.mark.parametrize("field,value", [("dim", 4), ("nx", 2), ("nghost", 2), ("dx", 0.0),
                                         ("dt", float("nan")), ("bc_y", 7)])
def test_params_check_rejects(lsgb_mod, field, value):
    p = lsgb_mod.params(3, 8, 8, 8)
    setattr(p, field, value)
    with pytest.raises(lsgb_mod.LsgbError) as e:
        lsgb_mod.check_params(p)
    assert e.value.code == 1 and str(e.value)


def test_reinit_params_checked_only_when_enabled(lsgb_mod):
    p = lsgb_mod.params(2, 8, 8, reinit_interval=0)
    lsgb_mod.check_params(p)
    p.enable_reinit = 1
    with pytest.raises(lsgb_mod.LsgbError):
        lsgb_mod.check_params(p)


def test_cfl_dt_matches_oracle(lsgb_mod, port):
    from oracle import Problem
    for dim, ms, sl in ((3, 1.7, 0.2), (2, 0.0, 0.0), (3, 0.0, 0.3)):
        p = lsgb_mod.params(dim, 32, 16, 8, s_l=sl, cfl=0.5)
        pb = Problem(nx=32, ny=16, nz=8, dim=dim, s_l=sl)
        assert lsgb_mod.cfl_dt(p, ms) == port.cfl_dt(pb, 0.5, ms)


def test_null_and_bad_arguments_fail_cleanly(lsgb_mod):
    L = lsgb_mod.lib()
    assert L.lsgb_params_check(None) == 1
    assert b"NULL" in L.lsgb_last_error()
    p = lsgb_mod.params(3, 8, 8, 8)
    # NULL device pointers are rejected before any CUDA call
    rc = L.lsgb_rk3_step_f64(C.byref(p), None, None, None, None, None, None, None, None, None)
    assert rc == 1
    assert L.lsgb_solver_advance(None, 1) == 1


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU failure path")
def test_solver_create_fails_loudly_without_gpu(lsgb_mod):
    with pytest.raises(lsgb_mod.LsgbError) as e:
        lsgb_mod.Solver(lsgb_mod.params(3, 8, 8, 8))
    assert e.value.code in (2, 3)
