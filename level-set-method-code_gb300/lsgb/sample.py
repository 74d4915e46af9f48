"""The reference's sample surface (sample/field.hpp, sample/weno5_rk3.hpp):
2D Field2D arrays with the local Lax-Friedrichs G-equation scheme, anchored +
periodic boundaries, first-order reinitialisation, and the forced Bunsen-flame
time loop of sample/main.cpp -- as ctypes calls into the CUDA library
(lsgb_sample_* in include/lsgb.h).

Arrays are float64 CUDA tensors of shape (ny+6, nx+6) (Field2D::data's
element order); ``run`` takes a stack of shape (n_inst, ny+6, nx+6), one
instance per forcing frequency.  There is no CPU path.

The workload constants of sample/config.hpp are kept as defaults.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _check, _stream, lib

# sample/config.hpp
NX = NY = 800
LX = LY = 0.02
DT = 0.0000025
FINAL_TIME = 0.16
SL = 0.4
U0, V0 = 0.0, 0.8
EPS_U = EPS_V = 0.05


class Forcing(C.Structure):
    """Mirror of ``lsgb_sample_forcing``."""

    _fields_ = [("u0", C.c_double), ("v0", C.c_double), ("eps_u", C.c_double), ("eps_v", C.c_double)]


def spacing(nx: int = NX, ny: int = NY, lx: float = LX, ly: float = LY):
    """DX = LX / (NX - 1), DY = LY / (NY - 1) (sample/config.hpp:8-9)."""
    return lx / (nx - 1), ly / (ny - 1)


def bunsen(nx: int = NX, ny: int = NY, lx: float = LX, ly: float = LY, R: float = 0.005,
           flame_angle: float = 30.0, X0: float = 0.01, Y0: float = 0.0) -> np.ndarray:
    """Initial G of sample/main.cpp:95-116 on every cell of the (ny+6, nx+6)
    array: minus the signed distance to a Bunsen cone of half-width R at x = X0,
    cone angle flame_angle, base at y = Y0; x = (i-3) DX, y = (j-3) DY."""
    dx, dy = spacing(nx, ny, lx, ly)
    slope = math.tan((90.0 - flame_angle) * math.pi / 180.0)
    j, i = np.meshgrid(np.arange(ny + 6), np.arange(nx + 6), indexing="ij")
    x = (i - 3) * dx
    y = (j - 3) * dy
    d = np.where(x < X0, slope * (x - (X0 - R)) - (y - Y0), -slope * (x - (X0 + R)) - (y - Y0))
    return np.ascontiguousarray(-d)


def _p(t):
    if not (getattr(t, "is_cuda", False) and str(t.dtype) == "torch.float64" and t.is_contiguous()):
        raise ValueError("the sample surface wants contiguous float64 CUDA tensors")
    return C.c_void_p(t.data_ptr())


def _dims(G):
    return G.shape[-1] - 6, G.shape[-2] - 6


def rhs(G, u, v, dx: float, dy: float, S_L: float, out=None, stream=None):
    """compute_geqn_rhs: -H on the interior, zero ghosts."""
    import torch
    nx, ny = _dims(G)
    if out is None:
        out = torch.empty_like(G)
    _check(lib().lsgb_sample_rhs(nx, ny, _p(G), _p(u), _p(v), _p(out), C.c_double(dx), C.c_double(dy),
                                 C.c_double(S_L), _stream(stream)))
    return out


def rk3_step(G, u, v, dx: float, dy: float, dt: float, S_L: float, G_initial, stream=None):
    """RK3_step, in place on G."""
    nx, ny = _dims(G)
    _check(lib().lsgb_sample_rk3_step(nx, ny, _p(G), _p(u), _p(v), C.c_double(dx), C.c_double(dy),
                                      C.c_double(dt), C.c_double(S_L), _p(G_initial), None, _stream(stream)))
    return G


def first_order_upwind(G, u, v, dx: float, dy: float, dt: float, S_L: float, stream=None):
    """compute_first_order_upwind, in place on G."""
    nx, ny = _dims(G)
    _check(lib().lsgb_sample_first_order_upwind(nx, ny, _p(G), _p(u), _p(v), C.c_double(dx), C.c_double(dy),
                                                C.c_double(dt), C.c_double(S_L), None, _stream(stream)))
    return G


def apply_periodic(G, stream=None):
    nx, ny = _dims(G)
    _check(lib().lsgb_sample_apply_periodic(nx, ny, _p(G), _stream(stream)))
    return G


def apply_anchored_bc(G, G_initial, stream=None):
    nx, ny = _dims(G)
    _check(lib().lsgb_sample_apply_anchored_bc(nx, ny, _p(G), _p(G_initial), _stream(stream)))
    return G


def reinitialize(G, G_initial, dx: float, dy: float, num_iters: int, stream=None):
    nx, ny = _dims(G)
    _check(lib().lsgb_sample_reinitialize(nx, ny, _p(G), _p(G_initial), C.c_double(dx), C.c_double(dy),
                                          int(num_iters), None, _stream(stream)))
    return G


def run(G, G_initial, n_steps: int, dx: float, dy: float, freq, t=None, dt: float = DT, S_L: float = SL,
        u0: float = U0, v0: float = V0, eps_u: float = EPS_U, eps_v: float = EPS_V, stream=None):
    """The forced time loop of sample/main.cpp for n_steps steps on a stack
    G of shape (n_inst, ny+6, nx+6), instance q forced at freq[q] Hz from time
    t[q] (default 0).  G_initial: (ny+6, nx+6) shared, or one per instance.
    Returns the new times."""
    nx, ny = _dims(G)
    n_inst = 1 if G.dim() == 2 else G.shape[0]
    freq_a = (C.c_int * n_inst)(*[int(f) for f in freq])
    t_a = (C.c_double * n_inst)(*([0.0] * n_inst if t is None else [float(x) for x in t]))
    shared = 1 if G_initial.dim() == 2 else 0
    f = Forcing(u0, v0, eps_u, eps_v)
    _check(lib().lsgb_sample_run(n_inst, nx, ny, int(n_steps), _p(G), _p(G_initial), shared, C.c_double(dx),
                                 C.c_double(dy), C.c_double(dt), C.c_double(S_L), C.byref(f), freq_a, t_a, None,
                                 _stream(stream)))
    return list(t_a)
