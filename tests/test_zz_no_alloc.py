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


class _Driver:
    """The CUDA driver API through ctypes (libcuda.so.1, present wherever a
    GPU is): the device's default memory pool, which cudaMallocAsync draws
    on, and the device's free memory, which cudaMalloc reduces."""

    USED_MEM_CURRENT, USED_MEM_HIGH = 7, 8  # CUmemPool_attribute

    def __init__(self, ordinal: int):
        self.L = C.CDLL("libcuda.so.1")
        assert self.L.cuInit(0) == 0
        dev = C.c_int()
        assert self.L.cuDeviceGet(C.byref(dev), ordinal) == 0
        self.pool = C.c_void_p()
        assert self.L.cuDeviceGetDefaultMemPool(C.byref(self.pool), dev) == 0

    def pool_attr(self, attr: int) -> int:
        v = C.c_uint64()
        assert self.L.cuMemPoolGetAttribute(self.pool, attr, C.byref(v)) == 0
        return v.value

    def reset_high_watermark(self):
        zero = C.c_uint64(0)  # setting 0 resets the watermark to the current use
        assert self.L.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH, C.byref(zero)) == 0

    def free_bytes(self) -> int:
        free, total = C.c_size_t(), C.c_size_t()
        assert self.L.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
        return free.value


def test_noalloc_allocates_no_device_memory(cuda, lsgb_mod):
    """After its set-up call the entry point draws nothing from the stream-
    ordered pool (the pool's high watermark stays at its current use) and
    takes no device memory (the device's free memory is unchanged), while the
    allocating entry point's per-call scratch does raise the watermark."""
    import torch
    lib = lsgb_mod.lib()
    p = lsgb_mod.params(3, 64, 48, 40)
    G = torch.from_numpy(_fields(p.shape(), 3)).cuda()
    ref = _volume(lib, "lsgb_volume_f64", p, G)
    _volume(lib, "lsgb_volume_f64_noalloc", p, G)  # set-up call: looks the scratch address up
    torch.cuda.synchronize()
    drv = _Driver(torch.cuda.current_device())
    used = drv.pool_attr(drv.USED_MEM_CURRENT)
    drv.reset_high_watermark()
    free0 = drv.free_bytes()
    for _ in range(3):
        assert _volume(lib, "lsgb_volume_f64_noalloc", p, G)[1] == ref[1]
    assert drv.pool_attr(drv.USED_MEM_HIGH) == used
    assert drv.free_bytes() == free0
    _volume(lib, "lsgb_volume_f64", p, G)  # the measurement does see a per-call allocation
    assert drv.pool_attr(drv.USED_MEM_HIGH) > used


def test_noalloc_rejects_grids_beyond_its_scratch(cuda, lsgb_mod):
    import torch
    lib = lsgb_mod.lib()
    p = lsgb_mod.params(3, 1100, 1100, 1100)  # 1.33e9 interior cells > 2^30
    G = torch.zeros(8, dtype=torch.float64, device="cuda")  # never read: rejected first
    vol = C.c_double()
    rc = lib.lsgb_volume_f64_noalloc(C.byref(p), C.c_void_p(G.data_ptr()), C.byref(vol), None, None)
    assert rc == 1
    assert b"at most" in lib.lsgb_last_error()
