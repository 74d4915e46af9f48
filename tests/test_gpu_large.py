"""A grid of more than 2^31 cells (64-bit element offsets; needs a GB300).

The fields are invariant along z, so every z face difference is exactly
zero and each plane of a 1292^3 run (2.16e9 cells, the 64-bit-offset
instances of the stage, reinit and conversion kernels) must equal, bit for
bit, the planes of the same problem on 8 planes (32-bit offsets).  Periodic
in every direction; two RK3 steps with an HCR-2 reinitialisation after the
first.  About 125 GB of device memory at the peak.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1292  # 1292^3 = 2.1567e9 > 2^31 - 1; N % 4 == 0 keeps the bulk-tensor staging


def fields(torch, nz):
    x = torch.arange(N, dtype=torch.float64, device="cuda") / N
    Y, X = torch.meshgrid(x, x, indexing="ij")  # [ny, nx]
    G = torch.sqrt((X - 0.5) ** 2 + (Y - 0.45) ** 2) - 0.3
    u = 0.8 * torch.sin(2 * math.pi * Y) + 0.1
    v = -0.6 * torch.sin(2 * math.pi * X)
    w = torch.zeros_like(G)
    return [f.expand(nz, N, N).contiguous() for f in (G, u, v, w)]


def run(lsgb, torch, nz, steps):
    p = lsgb.params(3, N, N, nz, dx=1 / N, dy=1 / N, dz=1 / N, s_l=0.2, dt=2e-4, enable_reinit=True,
                    reinit_interval=1, reinit_iterations=2)
    s = lsgb.Solver(p, "f32")
    G, u, v, w = fields(torch, nz)
    torch.cuda.synchronize()
    s.set_fields(G, u, v, w, layout="compact")
    torch.cuda.synchronize()
    del u, v, w
    s.advance(steps)
    s.get_G(layout="compact", out=G)  # FP64 result into the input buffer
    torch.cuda.synchronize()
    s.close()
    return G


def test_over_2g_cells_equals_small_extrusion(cuda, lsgb_mod):
    import torch
    free, _ = torch.cuda.mem_get_info()
    if free < 140e9:
        pytest.skip(f"needs ~140 GB of free device memory, {free / 1e9:.0f} GB free")
    steps = 2
    small = run(lsgb_mod, torch, 8, steps)
    ref = small[0].clone()
    for k in range(small.shape[0]):
        assert torch.equal(small[k], ref)
    assert float((ref - fields(torch, 1)[0][0]).abs().max()) > 0  # the step moved the front
    del small
    big = run(lsgb_mod, torch, N, steps)
    bad = [k for k in range(N) if not torch.equal(big[k], ref)]
    assert not bad, f"{len(bad)} planes differ, first {bad[:5]}"
    assert np.isfinite(float(big.abs().max()))
