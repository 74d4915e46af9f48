"""Python binding of the GB300 level-set solver (ctypes over the C ABI).

The product is the CUDA library ``_build/liblsgb.so`` with the C ABI of
``include/lsgb.h``; this module only marshals arguments.  It never computes a
result itself and has no CPU fallback: if the library is missing or no GPU is
present, the calls fail with :class:`LsgbError`.

Arrays
  * host arrays: float64 numpy arrays;
  * device arrays: objects with ``data_ptr()`` and ``is_cuda`` (torch tensors);
  * ``layout="ghosted"`` is the reference's layout with 3 ghost cells per side,
    shape ``(nz+6, ny+6, nx+6)`` / ``(ny+6, nx+6)``; ``"compact"`` is the
    interior only, ``(nz, ny, nx)`` / ``(ny, nx)``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "_build", "liblsgb.so")

OK = 0
ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_NUMERIC, ERR_STATE, ERR_UNSUPPORTED = 1, 2, 3, 4, 5, 6
BC_PERIODIC, BC_ZERO_GRADIENT = 0, 1
PREC_F64, PREC_F32 = 0, 1
LAYOUT_GHOSTED, LAYOUT_COMPACT = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1
MAX_MODES = 32


class LsgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lsgb error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    """Mirror of ``lsgb_params`` (include/lsgb.h)."""

    _fields_ = [
        ("dim", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("nghost", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("s_l", C.c_double), ("dt", C.c_double), ("cfl", C.c_double), ("epsilon", C.c_double),
        ("enable_reinit", C.c_int), ("reinit_interval", C.c_int), ("reinit_iterations", C.c_int),
        ("reinit_dtau", C.c_double), ("reinit_beta", C.c_double),
        ("bc_x", C.c_int), ("bc_y", C.c_int), ("bc_z", C.c_int),
    ]

    def shape(self, layout: str = "ghosted"):
        g = 6 if layout == "ghosted" else 0
        if self.dim == 3:
            return (self.nz + g, self.ny + g, self.nx + g)
        return (self.ny + g, self.nx + g)

    @property
    def cells(self) -> int:
        return self.nx * self.ny * (self.nz if self.dim == 3 else 1)


class Synth(C.Structure):
    """Mirror of ``lsgb_synth`` (include/lsgb.h)."""

    _fields_ = [
        ("center", C.c_double * 3), ("r0", C.c_double),
        ("n_shape_modes", C.c_int),
        ("shape_l", C.c_int * MAX_MODES), ("shape_m", C.c_int * MAX_MODES),
        ("shape_amp", C.c_double * MAX_MODES),
        ("n_vel_modes", C.c_int),
        ("vel_k", (C.c_double * 3) * MAX_MODES), ("vel_c", (C.c_double * 3) * MAX_MODES),
        ("vel_phase", C.c_double * MAX_MODES), ("vel_scale", C.c_double),
    ]


_lib = None


def lib() -> C.CDLL:
    """Load liblsgb.so (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LsgbError(-1, f"{LIB_PATH} is missing: run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    L.lsgb_last_error.restype = C.c_char_p
    L.lsgb_version.restype = C.c_char_p
    L.lsgb_launch_count.restype = C.c_uint64
    _lib = L
    return L


def _check(rc: int):
    if rc != OK:
        raise LsgbError(rc, lib().lsgb_last_error().decode())


def version() -> str:
    return lib().lsgb_version().decode()


def launch_count() -> int:
    return int(lib().lsgb_launch_count())


def params(dim: int, nx: int, ny: int, nz: int = 1, **kw) -> Params:
    """Reference defaults (lsgb_params_default) with keyword overrides."""
    p = Params()
    lib().lsgb_params_default(C.byref(p), dim, nx, ny, nz if dim == 3 else 1)
    for k, v in kw.items():
        if k in ("bc_x", "bc_y", "bc_z") and isinstance(v, str):
            v = {"periodic": BC_PERIODIC, "zero_gradient": BC_ZERO_GRADIENT}[v]
        if not hasattr(p, k):
            raise AttributeError(k)
        setattr(p, k, int(v) if isinstance(v, bool) else v)
    if "reinit_dtau" not in kw and any(k in kw for k in ("dx", "dy", "dz")):
        h = min(p.dx, p.dy, p.dz) if dim == 3 else min(p.dx, p.dy)
        p.reinit_dtau = 0.25 * h
    return p


def check_params(p: Params):
    _check(lib().lsgb_params_check(C.byref(p)))


# -- pointer helpers --------------------------------------------------------
def _is_dev(a) -> bool:
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _ptr(a):
    if a is None:
        return None
    if _is_dev(a):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64 or not a.flags.c_contiguous:
            raise ValueError("host arrays must be C-contiguous float64")
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):  # torch CPU tensor (pinned host buffers)
        return C.c_void_p(a.data_ptr())
    raise TypeError(type(a))


def _mem(*arrs) -> int:
    kinds = {MEM_DEVICE if _is_dev(a) else MEM_HOST for a in arrs if a is not None}
    if len(kinds) > 1:
        raise ValueError("mix of host and device arrays")
    return kinds.pop() if kinds else MEM_HOST


def _layout(name: str) -> int:
    return {"ghosted": LAYOUT_GHOSTED, "compact": LAYOUT_COMPACT}[name]


def _stream(stream) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(0)
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


# -- drop-in FP64 entry points (device tensors, ghosted layout) -------------
def rk3_step_f64(p: Params, G_n, G_new, G_1, G_2, u, v, w=None, sl=None, stream=None):
    """lsgb_rk3_step_f64 -- rk3TimeStep3D / rk3TimeStep on device buffers."""
    _check(lib().lsgb_rk3_step_f64(C.byref(p), _ptr(G_n), _ptr(G_new), _ptr(G_1), _ptr(G_2),
                                   _ptr(u), _ptr(v), _ptr(w), _ptr(sl), _stream(stream)))


def apply_bc_f64(p: Params, G, stream=None):
    _check(lib().lsgb_apply_bc_f64(C.byref(p), _ptr(G), _stream(stream)))


def reinit_f64(p: Params, phi, phi_tmp, phi0, r_tilde, flag, stream=None):
    """lsgb_reinit_f64 -- reinitializeWithSwap[3D]; returns (phi, phi_tmp)
    after the swap (the tensors themselves, reordered)."""
    a = C.c_void_p(phi.data_ptr())
    b = C.c_void_p(phi_tmp.data_ptr())
    _check(lib().lsgb_reinit_f64(C.byref(p), C.byref(a), C.byref(b), _ptr(phi0), _ptr(r_tilde),
                                 _ptr(flag), _stream(stream)))
    if a.value == phi.data_ptr():
        return phi, phi_tmp
    return phi_tmp, phi


def volume_f64(p: Params, G, stream=None):
    vol = C.c_double()
    cnt = C.c_int64()
    _check(lib().lsgb_volume_f64(C.byref(p), _ptr(G), C.byref(vol), C.byref(cnt), _stream(stream)))
    return vol.value, cnt.value


def l2_error_f64(p: Params, G, G_ref, stream=None) -> float:
    r = C.c_double()
    _check(lib().lsgb_l2_error_f64(C.byref(p), _ptr(G), _ptr(G_ref), C.byref(r), _stream(stream)))
    return r.value


def max_speed_f64(p: Params, u, v, w=None, stream=None) -> float:
    r = C.c_double()
    _check(lib().lsgb_max_speed_f64(C.byref(p), _ptr(u), _ptr(v), _ptr(w), C.byref(r), _stream(stream)))
    return r.value


def cfl_dt(p: Params, max_speed: float) -> float:
    r = C.c_double()
    _check(lib().lsgb_cfl_dt(C.byref(p), C.c_double(max_speed), C.byref(r)))
    return r.value


# -- solver handle ------------------------------------------------------------
class Solver:
    """Device-resident solver (lsgb_solver_*)."""

    def __init__(self, p: Params, precision: str = "f64"):
        self._h = C.c_void_p()
        prec = {"f64": PREC_F64, "f32": PREC_F32}[precision]
        _check(lib().lsgb_solver_create(C.byref(p), prec, C.byref(self._h)))
        self.precision = precision
        self.p = self.params()

    def close(self):
        if self._h:
            lib().lsgb_solver_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def params(self) -> Params:
        p = Params()
        _check(lib().lsgb_solver_get_params(self._h, C.byref(p)))
        return p

    def set_stream(self, stream):
        _check(lib().lsgb_solver_set_stream(self._h, _stream(stream)))

    def set_dt(self, dt: float):
        _check(lib().lsgb_solver_set_dt(self._h, C.c_double(dt)))

    def set_fields(self, G=None, u=None, v=None, w=None, layout: str = "ghosted"):
        _check(lib().lsgb_solver_set_fields(self._h, _ptr(G), _ptr(u), _ptr(v), _ptr(w),
                                            _layout(layout), _mem(G, u, v, w)))

    def set_sl_field(self, sl, layout: str = "ghosted"):
        _check(lib().lsgb_solver_set_sl_field(self._h, _ptr(sl), _layout(layout), _mem(sl)))

    def get_G(self, layout: str = "ghosted", out=None):
        p = self.params()
        if out is None:
            out = np.empty(p.shape(layout), dtype=np.float64)
        _check(lib().lsgb_solver_get_G(self._h, _ptr(out), _layout(layout), _mem(out)))
        return out

    def advance(self, n_steps: int):
        _check(lib().lsgb_solver_advance(self._h, int(n_steps)))

    def reinit(self):
        _check(lib().lsgb_solver_reinit(self._h))

    @property
    def step(self) -> int:
        s = C.c_int()
        _check(lib().lsgb_solver_get_step(self._h, C.byref(s)))
        return s.value

    @step.setter
    def step(self, v: int):
        _check(lib().lsgb_solver_set_step(self._h, int(v)))

    def volume(self):
        vol = C.c_double()
        cnt = C.c_int64()
        _check(lib().lsgb_solver_volume(self._h, C.byref(vol), C.byref(cnt)))
        return vol.value, cnt.value

    def max_speed(self) -> float:
        r = C.c_double()
        _check(lib().lsgb_solver_max_speed(self._h, C.byref(r)))
        return r.value

    def compute_dt(self, cfl: float) -> float:
        r = C.c_double()
        _check(lib().lsgb_solver_compute_dt(self._h, C.c_double(cfl), C.byref(r)))
        return r.value

    def l2_error(self, G_ref, layout: str = "ghosted") -> float:
        r = C.c_double()
        _check(lib().lsgb_solver_l2_error(self._h, _ptr(G_ref), _layout(layout), _mem(G_ref), C.byref(r)))
        return r.value

    def run_host(self, G, u, v, w, n_steps: int, out, layout: str = "ghosted"):
        _check(lib().lsgb_solver_run_host(self._h, _ptr(G), _ptr(u), _ptr(v), _ptr(w), int(n_steps),
                                          _ptr(out), _layout(layout)))
        return out

    def synth(self, d: Synth):
        _check(lib().lsgb_solver_synth(self._h, C.byref(d)))


def _set_velocity_deformation(self, t: float, T: float):
    """Device-side deformation vortex of the reference's default 3D case."""
    _check(lib().lsgb_solver_set_velocity_deformation(self._h, C.c_double(t), C.c_double(T)))


def _set_velocity_deformation_live(self, t: float, T: float):
    """Live deformation vortex: every step of advance() uses the vortex at the
    handle's time (starting at t, advancing by dt per step)."""
    _check(lib().lsgb_solver_set_velocity_deformation_live(self._h, C.c_double(t), C.c_double(T)))


def _time(self) -> float:
    """Live-mode time: the t of the next step."""
    t = C.c_double()
    _check(lib().lsgb_solver_get_time(self._h, C.byref(t)))
    return t.value


Solver.set_velocity_deformation = _set_velocity_deformation
Solver.set_velocity_deformation_live = _set_velocity_deformation_live
Solver.time = _time


def _get_field(self, which: str, layout: str = "ghosted", out=None):
    """Download a resident field ("G", "u", "v", "w", "sl") as FP64."""
    code = {"G": 0, "u": 1, "v": 2, "w": 3, "sl": 4}[which]
    p = self.params()
    if out is None:
        out = np.empty(p.shape(layout), dtype=np.float64)
    _check(lib().lsgb_solver_get_field(self._h, code, _ptr(out), _layout(layout), _mem(out)))
    return out


def _enable_timing(self, on: bool = True):
    _check(lib().lsgb_solver_enable_timing(self._h, int(on)))


def _kernel_times(self):
    """(stage_ms, stage_launches, reinit_ms, reinit_launches) since enable_timing."""
    a, b = C.c_double(), C.c_double()
    na, nb = C.c_int64(), C.c_int64()
    _check(lib().lsgb_solver_kernel_times(self._h, C.byref(a), C.byref(na), C.byref(b), C.byref(nb)))
    return a.value, na.value, b.value, nb.value


Solver.get_field = _get_field
Solver.enable_timing = _enable_timing
Solver.kernel_times = _kernel_times


def _set_tile(self, tile: int):
    _check(lib().lsgb_solver_set_tile(self._h, int(tile)))


def _get_tile(self) -> int:
    t = C.c_int()
    _check(lib().lsgb_solver_get_tile(self._h, C.byref(t)))
    return t.value


def _autotune(self, reps: int = 3):
    """Pick the fastest tile shape for this grid (lsgb_solver_autotune)."""
    t = C.c_int()
    ms = C.c_float()
    _check(lib().lsgb_solver_autotune(self._h, int(reps), C.byref(t), C.byref(ms)))
    return t.value, ms.value


def _debug_drop_copies(self, on: bool):
    """Test hook: the TMA-fed FP32 3D stage kernel issues no bulk copies, so
    its bounded waits time out and the next synchronising call raises."""
    _check(lib().lsgb_solver_debug_drop_copies(self._h, int(bool(on))))


Solver.debug_drop_copies = _debug_drop_copies
Solver.set_tile = _set_tile
Solver.get_tile = _get_tile
Solver.autotune = _autotune


class _Borrowed(Solver):
    """Solver handle owned by a Batch (not destroyed by Python)."""

    def __init__(self, handle):
        self._h = handle
        self.precision = None
        self.p = self.params()

    def close(self):
        self._h = C.c_void_p()


class Batch:
    """Many independent instances advanced together (lsgb_batch_*)."""

    def __init__(self, precision: str = "f32", lanes: int = 16):
        self._h = C.c_void_p()
        prec = {"f64": PREC_F64, "f32": PREC_F32}[precision]
        _check(lib().lsgb_batch_create(prec, int(lanes), C.byref(self._h)))
        self.instances = []

    def add(self, p: Params) -> Solver:
        h = C.c_void_p()
        idx = C.c_int()
        _check(lib().lsgb_batch_add(self._h, C.byref(p), C.byref(h), C.byref(idx)))
        s = _Borrowed(h)
        self.instances.append(s)
        return s

    def autotune(self, reps: int = 3):
        _check(lib().lsgb_batch_autotune(self._h, int(reps)))

    def advance(self, n_steps: int):
        _check(lib().lsgb_batch_advance(self._h, int(n_steps)))

    def sync(self):
        _check(lib().lsgb_batch_sync(self._h))

    def stats(self):
        a, b = C.c_int64(), C.c_int64()
        _check(lib().lsgb_batch_stats(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_mode(self, mode: str):
        """"grouped" (one launch per stage for all instances of a
        dimensionality; FP32) or "lanes" (per-instance launches on streams)."""
        _check(lib().lsgb_batch_set_mode(self._h, {"grouped": 0, "lanes": 1}[mode]))

    @property
    def mode(self) -> str:
        m = C.c_int()
        _check(lib().lsgb_batch_get_mode(self._h, C.byref(m)))
        return "grouped" if m.value == 0 else "lanes"

    def stream_handle(self) -> int:
        p = C.c_void_p()
        _check(lib().lsgb_batch_stream(self._h, C.byref(p)))
        return p.value or 0

    def close(self):
        if self._h:
            for s in self.instances:
                s.close()
            lib().lsgb_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Adjoint:
    """Discrete adjoint of a solver's steps (lsgb_adjoint_*).

    ``forward(n)`` advances the solver with checkpoints every
    ``checkpoint_interval`` steps; ``backward(dL_dGT)`` (or the seed stored by
    ``loss(seed=True)``) runs the reverse sweep; ``grad(name)`` returns
    dL/d(name) for name in "G0", "sl", "u", "v", "w".  Destroy it before its
    solver."""

    _CODES = {"G0": 0, "u": 1, "v": 2, "w": 3, "sl": 4}

    def __init__(self, solver: Solver, checkpoint_interval: int = 20):
        self._h = C.c_void_p()
        self.solver = solver
        _check(lib().lsgb_adjoint_create(solver._h, int(checkpoint_interval), C.byref(self._h)))

    def close(self):
        if self._h:
            lib().lsgb_adjoint_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_grads(self, sl: bool = True, velocity: bool = True):
        """Which parameter gradients the backward accumulates (dL/dG0 always)."""
        _check(lib().lsgb_adjoint_set_grads(self._h, (1 if sl else 0) | (2 if velocity else 0)))

    def set_slab(self, planes: int = 0):
        """z planes per slab of the 3D stage transpose (0 = automatic)."""
        _check(lib().lsgb_adjoint_set_slab(self._h, int(planes)))

    def forward(self, n_steps: int):
        _check(lib().lsgb_adjoint_forward(self._h, int(n_steps)))

    def set_target(self, G_target, eps: float, layout: str = "ghosted"):
        _check(lib().lsgb_adjoint_set_target(self._h, _ptr(G_target), _layout(layout), _mem(G_target),
                                             C.c_double(eps)))

    def loss(self, seed: bool = False) -> float:
        r = C.c_double()
        _check(lib().lsgb_adjoint_loss(self._h, int(seed), C.byref(r)))
        return r.value

    def backward(self, dL_dGT=None, layout: str = "ghosted"):
        _check(lib().lsgb_adjoint_backward(self._h, _ptr(dL_dGT), _layout(layout), _mem(dL_dGT)))

    def grad(self, which: str = "sl", layout: str = "compact", out=None):
        p = self.solver.params()
        if out is None:
            out = np.empty(p.shape(layout), dtype=np.float64)
        _check(lib().lsgb_adjoint_get_grad(self._h, self._CODES[which], _ptr(out), _layout(layout), _mem(out)))
        return out


# -- binary dumps (the reference's .bin format) --------------------------------
def dump_bytes(p: Params) -> int:
    n = C.c_size_t()
    _check(lib().lsgb_dump_bytes(C.byref(p), C.byref(n)))
    return n.value


def dump_f64(p: Params, G, stream=None) -> bytes:
    """Image of a ghosted FP64 device array (saveFieldBinary3D / saveFieldBinary)."""
    buf = np.empty(dump_bytes(p), dtype=np.uint8)
    _check(lib().lsgb_dump_f64(C.byref(p), _ptr(G), C.c_void_p(buf.ctypes.data), MEM_HOST, _stream(stream)))
    return buf.tobytes()


def read_dump(data, dim: int):
    """(header ints, ghosted array) of a dump image or file (3D header
    {nx, ny, nz, nghost}, 2D {nx, ny, nghost})."""
    if isinstance(data, (str, os.PathLike)):
        with open(data, "rb") as f:
            data = f.read()
    nh = 4 if dim == 3 else 3
    h = np.frombuffer(data, dtype=np.int32, count=nh)
    g = int(h[-1])
    shape = (int(h[2]) + 2 * g, int(h[1]) + 2 * g, int(h[0]) + 2 * g) if dim == 3 else (int(h[1]) + 2 * g, int(h[0]) + 2 * g)
    arr = np.frombuffer(data, dtype=np.float64, offset=4 * nh).reshape(shape)
    return [int(x) for x in h], arr


def _solver_dump(self) -> bytes:
    buf = np.empty(dump_bytes(self.params()), dtype=np.uint8)
    _check(lib().lsgb_solver_dump(self._h, C.c_void_p(buf.ctypes.data), MEM_HOST))
    return buf.tobytes()


def _solver_snapshot(self, path: str):
    """Write the current G's dump to `path` in the background."""
    _check(lib().lsgb_solver_snapshot(self._h, os.fsencode(path)))


def _solver_snapshot_wait(self):
    _check(lib().lsgb_solver_snapshot_wait(self._h))


Solver.dump = _solver_dump
Solver.snapshot = _solver_snapshot
Solver.snapshot_wait = _solver_snapshot_wait


class Diagnostics(C.Structure):
    """Mirror of ``lsgb_diagnostics`` (analyze_error.m's quantities)."""

    _fields_ = [(n, C.c_double) for n in ("l2", "linf", "l2_rel", "volume", "volume_ref", "volume_smooth",
                                          "volume_smooth_ref", "grad_mean", "grad_std", "iface_mean",
                                          "iface_max")] + [("band_cells", C.c_int64), ("iface_points", C.c_int64),
                                                           ("contour_hausdorff", C.c_double),
                                                           ("contour_mean", C.c_double),
                                                           ("contour_points", C.c_int64),
                                                           ("contour_points_ref", C.c_int64)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


def _solver_diagnostics(self, G_ref, layout: str = "ghosted") -> dict:
    """Error / conservation diagnostics of G against G_ref (FP64)."""
    d = Diagnostics()
    _check(lib().lsgb_solver_diagnostics(self._h, _ptr(G_ref), _layout(layout), _mem(G_ref), C.byref(d)))
    return d.as_dict()


Solver.diagnostics = _solver_diagnostics
