"""lsgb_volume_f64_noalloc: the interface-volume reduction for callers that
cannot let the library allocate device memory during the call (their own pool
already holds the device, or the call sits on a path that may not block in
the allocator).  It must give what lsgb_volume_f64 gives, through the C ABI,
on consecutive calls that share its one fixed scratch array.

This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(shape, seed):
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(rng.standard_normal(shape) * 0.1 - 0.02)


def _volume(lib, fn, p, G):
    vol = C.c_double()
    cnt = C.c_int64()
    rc = getattr(lib, fn)(C.byref(p), C.c_void_p(G.data_ptr()), C.byref(vol), C.byref(cnt), None)
    assert rc == 0, lib.lsgb_last_error()
    return vol.value, cnt.value


@pytest.mark.parametrize("dim,n", [(3, (37, 29, 23)), (2, (300, 257, 1))])
def test_noalloc_volume_matches_allocating_entry_point(cuda, lsgb_mod, dim, n):
    import torch
    lib = lsgb_mod.lib()
    p = lsgb_mod.params(dim, *n)
    results = []
    for seed in (1, 2):  # two calls in a row through the shared scratch
        G = torch.from_numpy(_fields(p.shape(), seed)).cuda()
        ref = _volume(lib, "lsgb_volume_f64", p, G)
        got = _volume(lib, "lsgb_volume_f64_noalloc", p, G)
        assert got[1] == ref[1]
        assert got[0] == pytest.approx(ref[0], rel=1e-12)
        results.append(got)
    assert results[0][1] != results[1][1]  # the second call did not reuse the first result


def test_noalloc_rejects_grids_beyond_its_scratch(cuda, lsgb_mod):
    import torch
    lib = lsgb_mod.lib()
    p = lsgb_mod.params(3, 1100, 1100, 1100)  # 1.33e9 interior cells > 2^30
    G = torch.zeros(8, dtype=torch.float64, device="cuda")  # never read: rejected first
    vol = C.c_double()
    rc = lib.lsgb_volume_f64_noalloc(C.byref(p), C.c_void_p(G.data_ptr()), C.byref(vol), None, None)
    assert rc == 1
    assert b"at most" in lib.lsgb_last_error()
