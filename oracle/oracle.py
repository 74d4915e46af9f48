"""CPU oracles for the level-set hot path -- test infrastructure only.

Two interchangeable back ends with the same Python surface:

* ``kind="port"``: ``oracle/_build/liboracle.so``, the plain-C restatement in
  ``oracle/ls_oracle.c`` (built here and on any host by :func:`build_port`);
* ``kind="ref"``: ``oracle/_ref/libref{2d,3d}.so``, the reference's own CPU
  solver headers compiled unmodified by ``oracle/build_ref.sh`` (only where the
  reference source tree is present).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline and
reference legs import this module.  The product library never does.

All arrays are float64 numpy arrays in the reference's ghosted layout
(``[nz+6, ny+6, nx+6]`` in 3D, ``[ny+6, nx+6]`` in 2D, C order), exactly the
index map ``k*nxT*nyT + j*nxT + i`` of Local_code/level-set_MPI_3D/include/config.h:301-306.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
PORT_LIB = os.path.join(BUILD_DIR, "liboracle.so")


class OrcParams(C.Structure):
    """Mirror of ``orc_params`` in oracle/oracle_params.h."""

    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("dt", C.c_double), ("s_l", C.c_double), ("epsilon", C.c_double),
        ("enable_reinit", C.c_int), ("reinit_interval", C.c_int),
        ("reinit_iterations", C.c_int),
        ("reinit_dtau", C.c_double), ("reinit_beta", C.c_double),
        ("periodic_y", C.c_int),
    ]


@dataclass
class Problem:
    """Grid + physics of one run, with the reference's defaults
    (Local_code/level-set_MPI_3D/include/config.h:88-107)."""

    nx: int
    ny: int
    nz: int = 1
    dx: float = 0.0
    dy: float = 0.0
    dz: float = 0.0
    dt: float = 1e-3
    s_l: float = 0.0
    epsilon: float = 1e-10
    enable_reinit: bool = False
    reinit_interval: int = 10
    reinit_iterations: int = 2
    reinit_dtau: float = 0.0
    reinit_beta: float = 0.5
    periodic_y: bool = True
    dim: int = 3

    def __post_init__(self):
        if self.dx == 0.0:
            self.dx = 1.0 / self.nx
        if self.dy == 0.0:
            self.dy = 1.0 / self.ny
        if self.dz == 0.0:
            self.dz = 1.0 / self.nz if self.dim == 3 else self.dx
        if self.reinit_dtau == 0.0:
            h = min(self.dx, self.dy, self.dz) if self.dim == 3 else min(self.dx, self.dy)
            self.reinit_dtau = 0.25 * h

    @property
    def shape(self):
        if self.dim == 3:
            return (self.nz + 6, self.ny + 6, self.nx + 6)
        return (self.ny + 6, self.nx + 6)

    def c(self) -> OrcParams:
        return OrcParams(self.nx, self.ny, self.nz if self.dim == 3 else 1,
                         self.dx, self.dy, self.dz, self.dt, self.s_l, self.epsilon,
                         int(self.enable_reinit), self.reinit_interval, self.reinit_iterations,
                         self.reinit_dtau, self.reinit_beta, int(self.periodic_y))


def build_port(force: bool = False) -> str:
    """Compile oracle/ls_oracle.c and oracle/ls_oracle_sample.c into
    oracle/_build/liboracle.so (gcc, OpenMP, no FP contraction so every
    operation is the plain IEEE double op)."""
    srcs = [os.path.join(HERE, "ls_oracle.c"), os.path.join(HERE, "ls_oracle_sample.c")]
    os.makedirs(BUILD_DIR, exist_ok=True)
    deps = srcs + [os.path.join(HERE, "oracle_params.h")]
    if not force and os.path.exists(PORT_LIB) and all(os.path.getmtime(PORT_LIB) >= os.path.getmtime(d) for d in deps):
        return PORT_LIB
    tmp = PORT_LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-I", HERE, *srcs, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, PORT_LIB)
    return PORT_LIB


def build_ref(reference_root: str | None = None) -> bool:
    """Compile the reference's own solver headers (oracle/build_ref.sh) from
    the reference tree at ``reference_root`` (or ``$LSGB_REFERENCE_ROOT``).
    Returns False when no root is given or the tree is absent there."""
    env = dict(os.environ)
    root = reference_root or env.get("LSGB_REFERENCE_ROOT")
    if not root or not os.path.isdir(os.path.join(root, "Local_code")):
        return False
    env["LSGB_REFERENCE_ROOT"] = root
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True, env=env,
                   stdout=subprocess.DEVNULL)
    return True


def ref_available() -> bool:
    return (os.path.exists(os.path.join(REF_DIR, "libref3d.so"))
            and os.path.exists(os.path.join(REF_DIR, "libref2d.so")))


_DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_IP = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """Uniform wrapper over the port and the compiled reference."""

    def __init__(self, kind: str = "port"):
        self.kind = kind
        if kind == "port":
            lib = C.CDLL(build_port())
            self._l3 = self._l2 = lib
            self._p3, self._p2 = "orc3d_", "orc2d_"
            lib.orc3d_volume.restype = C.c_double
            lib.orc2d_area.restype = C.c_double
            lib.orc_l2.restype = C.c_double
            lib.orc_max_speed.restype = C.c_double
            lib.orc_cfl_dt.restype = C.c_double
        elif kind == "ref":
            if not ref_available():
                raise RuntimeError("oracle/_ref not built (reference tree absent?)")
            self._l3 = C.CDLL(os.path.join(REF_DIR, "libref3d.so"))
            self._l2 = C.CDLL(os.path.join(REF_DIR, "libref2d.so"))
            self._p3, self._p2 = "ref3d_", "ref2d_"
            self._l3.ref3d_volume.restype = C.c_double
            self._l3.ref3d_l2.restype = C.c_double
            self._l2.ref2d_area.restype = C.c_double
            self._l2.ref2d_l2.restype = C.c_double
        else:
            raise ValueError(kind)

    # -- helpers -----------------------------------------------------------
    def _f(self, pb: Problem, name: str):
        if pb.dim == 3:
            return getattr(self._l3, self._p3 + name)
        return getattr(self._l2, self._p2 + name)

    @staticmethod
    def _chk(pb: Problem, *arrs):
        for a in arrs:
            if a is None:
                continue
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.shape == pb.shape, \
                (a.dtype, a.shape, pb.shape)

    # -- hot path ------------------------------------------------------------
    def rk3_step(self, pb: Problem, G, u, v, w=None, sl=None):
        """One rk3TimeStep[3D]; returns the new ghosted field (input untouched)."""
        self._chk(pb, G, u, v, w, sl)
        Gn = G.copy()
        out = np.zeros_like(G)
        G1, G2, R = np.zeros_like(G), np.zeros_like(G), np.zeros_like(G)
        p = pb.c()
        if self.kind == "ref":
            assert sl is None, "the reference has no per-cell flame speed"
            if pb.dim == 3:
                self._l3.ref3d_rk3_step(C.byref(p), _ptr(Gn), _ptr(out), _ptr(G1), _ptr(G2), _ptr(R),
                                        _ptr(u), _ptr(v), _ptr(w))
            else:
                self._l2.ref2d_rk3_step(C.byref(p), _ptr(Gn), _ptr(out), _ptr(G1), _ptr(G2), _ptr(R),
                                        _ptr(u), _ptr(v))
        else:
            if pb.dim == 3:
                self._l3.orc3d_rk3_step(C.byref(p), _ptr(Gn), _ptr(out), _ptr(G1), _ptr(G2), _ptr(R),
                                        _ptr(u), _ptr(v), _ptr(w), _ptr(sl))
            else:
                self._l2.orc2d_rk3_step(C.byref(p), _ptr(Gn), _ptr(out), _ptr(G1), _ptr(G2), _ptr(R),
                                        _ptr(u), _ptr(v), _ptr(sl))
        return out

    def rhs(self, pb: Problem, G, u, v, w=None, sl=None):
        self._chk(pb, G, u, v, w, sl)
        R = np.zeros_like(G)
        p = pb.c()
        if self.kind == "ref":
            assert sl is None
            if pb.dim == 3:
                self._l3.ref3d_rhs(C.byref(p), _ptr(G), _ptr(R), _ptr(u), _ptr(v), _ptr(w))
            else:
                self._l2.ref2d_rhs(C.byref(p), _ptr(G), _ptr(R), _ptr(u), _ptr(v))
        else:
            if pb.dim == 3:
                self._l3.orc3d_rhs(C.byref(p), _ptr(G), _ptr(R), _ptr(u), _ptr(v), _ptr(w), _ptr(sl))
            else:
                self._l2.orc2d_rhs(C.byref(p), _ptr(G), _ptr(R), _ptr(u), _ptr(v), _ptr(sl))
        return R

    def apply_bc(self, pb: Problem, G):
        self._chk(pb, G)
        out = G.copy()
        self._f(pb, "apply_bc")(C.byref(pb.c()), _ptr(out))
        return out

    def reinit(self, pb: Problem, G):
        """reinitializeWithSwap[3D]; returns (phi, phi0, r_tilde, flag)."""
        self._chk(pb, G)
        phi = G.copy()
        tmp = np.zeros_like(G)
        phi0 = np.zeros_like(G)
        rt = np.zeros_like(G)
        flag = np.zeros(G.shape, dtype=np.int32)
        self._f(pb, "reinit")(C.byref(pb.c()), _ptr(phi), _ptr(tmp), _ptr(phi0), _ptr(rt),
                              flag.ctypes.data_as(C.POINTER(C.c_int)))
        return phi, phi0, rt, flag

    def run(self, pb: Problem, n_steps: int, G, u, v, w=None, sl=None, step0: int = 0):
        """Reference main loop with fixed velocity; returns the final field."""
        self._chk(pb, G, u, v, w, sl)
        out = G.copy()
        p = pb.c()
        if self.kind == "ref":
            assert sl is None and step0 == 0
            if pb.dim == 3:
                self._l3.ref3d_run(C.byref(p), n_steps, _ptr(out), _ptr(u), _ptr(v), _ptr(w))
            else:
                self._l2.ref2d_run(C.byref(p), n_steps, _ptr(out), _ptr(u), _ptr(v))
        else:
            if pb.dim == 3:
                rc = self._l3.orc3d_run(C.byref(p), n_steps, step0, _ptr(out), _ptr(u), _ptr(v), _ptr(w),
                                        _ptr(sl))
            else:
                rc = self._l2.orc2d_run(C.byref(p), n_steps, step0, _ptr(out), _ptr(u), _ptr(v), _ptr(sl))
            if rc != 0:
                raise MemoryError("oracle run: scratch allocation failed")
        return out

    def run_filled(self, pb: Problem, n_steps: int, G, u, v, w=None, sl=None, step0: int = 0):
        """:meth:`run` for grids too large for copies (the port only): G is
        advanced IN PLACE and u, v, w must already hold their boundary images
        (e.g. from :meth:`apply_bc`); they are read, not copied.  Scratch is 5
        fields + one int32 field.  Returns G."""
        assert self.kind == "port"
        self._chk(pb, G, u, v, w, sl)
        p = pb.c()
        if pb.dim == 3:
            rc = self._l3.orc3d_run_filled(C.byref(p), n_steps, step0, _ptr(G), _ptr(u), _ptr(v), _ptr(w),
                                           _ptr(sl))
        else:
            rc = self._l2.orc2d_run_filled(C.byref(p), n_steps, step0, _ptr(G), _ptr(u), _ptr(v), _ptr(sl))
        if rc != 0:
            raise MemoryError("oracle run: scratch allocation failed")
        return G

    # -- decision tape (3D port only): see the tape section of ls_oracle.c ----
    def tape(self, mode: str, stage=None, pseudo=None, flags=None):
        """mode "off", "record" or "replay"; stage / pseudo / flags are uint8
        arrays of shape (calls, nz * ny * nx) holding one row per rhs
        evaluation, HCR-2 pseudo-step and reinitialisation."""
        assert self.kind == "port"
        m = {"off": 0, "record": 1, "replay": 2}[mode]
        arrs = (stage, pseudo, flags)
        for a in arrs:
            assert a is None or (a.dtype == np.uint8 and a.flags.c_contiguous and a.ndim == 2)
        ptr = lambda a: None if a is None else a.ctypes.data_as(C.POINTER(C.c_ubyte))
        rows = lambda a: 0 if a is None else a.shape[0]
        self._l3.orc_tape_set(m, ptr(stage), C.c_long(rows(stage)), ptr(pseudo), C.c_long(rows(pseudo)),
                              ptr(flags), C.c_long(rows(flags)))
        self._tape_refs = arrs

    def tape_counts(self):
        """(rhs rows, pseudo-step rows, reinit rows used, overflow)."""
        out = (C.c_long * 4)()
        self._l3.orc_tape_counts(out)
        return tuple(int(x) for x in out)

    def volume(self, pb: Problem, G):
        """computeInterfaceVolume / computeInterfaceArea."""
        self._chk(pb, G)
        p = pb.c()
        if self.kind == "ref":
            if pb.dim == 3:
                return self._l3.ref3d_volume(C.byref(p), _ptr(G))
            return self._l2.ref2d_area(C.byref(p), _ptr(G))
        if pb.dim == 3:
            return self._l3.orc3d_volume(C.byref(p), _ptr(G), None)
        return self._l2.orc2d_area(C.byref(p), _ptr(G), None)

    def l2(self, pb: Problem, G, Gref):
        self._chk(pb, G, Gref)
        p = pb.c()
        if self.kind == "ref":
            if pb.dim == 3:
                return self._l3.ref3d_l2(C.byref(p), _ptr(G), _ptr(Gref))
            return self._l2.ref2d_l2(C.byref(p), _ptr(G), _ptr(Gref))
        return self._l3.orc_l2(C.byref(p), pb.dim, _ptr(G), _ptr(Gref))

    def max_speed(self, pb: Problem, u, v, w=None):
        assert self.kind == "port"
        return self._l3.orc_max_speed(C.byref(pb.c()), pb.dim, _ptr(u), _ptr(v), _ptr(w))

    def cfl_dt(self, pb: Problem, cfl: float, max_speed: float):
        assert self.kind == "port"
        return self._l3.orc_cfl_dt(C.byref(pb.c()), pb.dim, C.c_double(cfl), C.c_double(max_speed))

    def save_binary(self, pb: Problem, G, path: str):
        """The reference's own dump writer, saveFieldBinary3D / saveFieldBinary
        (io.h), on a ghosted array (ref only)."""
        assert self.kind == "ref"
        self._chk(pb, G)
        rc = self._f(pb, "save_binary")(C.byref(pb.c()), _ptr(G), path.encode())
        assert rc == 0, "reference dump writer failed"

    # -- reference-only end-to-end case ------------------------------------
    def deformation_test(self):
        """The reference's default 64^3 sphere-deformation run (ref only)."""
        assert self.kind == "ref"
        l2, v0, v1 = C.c_double(), C.c_double(), C.c_double()
        st = C.c_int()
        self._l3.ref3d_deformation_test(C.byref(l2), C.byref(v0), C.byref(v1), C.byref(st), None)
        return l2.value, v0.value, v1.value, st.value


    def zalesak_test(self, n: int):
        """The reference's 2D Zalesak known-answer run on n x n (ref only).
        Returns (G0, u, v, G_final) as ghosted (n+6, n+6) arrays and
        (l2, area0, area1, steps)."""
        assert self.kind == "ref"
        shape = (n + 6, n + 6)
        G0, u, v, Gf = (np.zeros(shape) for _ in range(4))
        out = np.zeros(4)
        self._l2.ref2d_zalesak(n, _ptr(G0), _ptr(u), _ptr(v), _ptr(Gf), _ptr(out))
        return G0, u, v, Gf, (float(out[0]), float(out[1]), float(out[2]), int(out[3]))


class SampleOracle:
    """The sample surface (sample/field.cpp, sample/weno5_rk3.cpp): 2D
    Field2D arrays as float64 numpy arrays of shape (ny+6, nx+6).

    ``kind="port"``: oracle/ls_oracle_sample.c (in liboracle.so);
    ``kind="ref"``: the reference's own sources compiled by build_ref.sh
    into oracle/_ref/libref_sample.so."""

    def __init__(self, kind: str = "port"):
        self.kind = kind
        if kind == "port":
            self._l = C.CDLL(build_port())
            self._p = "orcs_"
        elif kind == "ref":
            path = os.path.join(REF_DIR, "libref_sample.so")
            if not os.path.exists(path):
                raise RuntimeError("oracle/_ref/libref_sample.so not built (reference tree absent?)")
            self._l = C.CDLL(path)
            self._p = "refs_"
        else:
            raise ValueError(kind)

    def _fn(self, name):
        return getattr(self._l, self._p + name)

    @staticmethod
    def _dims(G):
        assert G.dtype == np.float64 and G.flags.c_contiguous and G.ndim == 2
        return G.shape[1] - 6, G.shape[0] - 6

    def rhs(self, G, u, v, dx, dy, S_L):
        nx, ny = self._dims(G)
        out = np.zeros_like(G)
        self._fn("rhs")(nx, ny, _ptr(G), _ptr(u), _ptr(v), _ptr(out), C.c_double(dx), C.c_double(dy),
                        C.c_double(S_L))
        return out

    def first_order_upwind(self, G, u, v, dx, dy, dt, S_L):
        nx, ny = self._dims(G)
        out = G.copy()
        self._fn("first_order_upwind")(nx, ny, _ptr(out), _ptr(u), _ptr(v), C.c_double(dx), C.c_double(dy),
                                       C.c_double(dt), C.c_double(S_L))
        return out

    def rk3_step(self, G, u, v, dx, dy, dt, S_L, G_initial):
        nx, ny = self._dims(G)
        out = G.copy()
        self._fn("rk3_step")(nx, ny, _ptr(out), _ptr(u), _ptr(v), C.c_double(dx), C.c_double(dy), C.c_double(dt),
                             C.c_double(S_L), _ptr(G_initial))
        return out

    def apply_periodic(self, G):
        nx, ny = self._dims(G)
        out = G.copy()
        self._fn("apply_periodic")(nx, ny, _ptr(out))
        return out

    def apply_anchored_bc(self, G, G_initial):
        nx, ny = self._dims(G)
        out = G.copy()
        self._fn("apply_anchored_bc")(nx, ny, _ptr(out), _ptr(G_initial))
        return out

    def reinitialize(self, G, G_initial, dx, dy, iters):
        nx, ny = self._dims(G)
        out = G.copy()
        self._fn("reinitialize")(nx, ny, _ptr(out), _ptr(G_initial), C.c_double(dx), C.c_double(dy), int(iters))
        return out

    def run(self, G, G_initial, n_steps, dx, dy, dt, S_L, u0, v0, eps_u, eps_v, freq, t0=0.0):
        """sample/main.cpp's time loop; returns (G, t)."""
        nx, ny = self._dims(G)
        out = G.copy()
        t = C.c_double(t0)
        self._fn("run")(nx, ny, int(n_steps), _ptr(out), _ptr(G_initial), C.c_double(dx), C.c_double(dy),
                        C.c_double(dt), C.c_double(S_L), C.c_double(u0), C.c_double(v0), C.c_double(eps_u),
                        C.c_double(eps_v), int(freq), C.byref(t))
        return out, t.value
