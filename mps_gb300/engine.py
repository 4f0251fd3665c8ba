"""ctypes binding of the engine's C ABI (include/mps_gb300.h).

This is the Python face of the same entry points a C/C++ caller binds; the
tests and bench.py drive the engine through it.  There is no fallback: if
the compiled library is missing or no sm_103 GPU is present, the calls
raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

(MPS_OK, MPS_ERR_ARG, MPS_ERR_CUDA, MPS_ERR_CAPACITY, MPS_ERR_TIMEOUT, MPS_ERR_NO_DEVICE,
 MPS_ERR_NONFINITE) = range(7)
FP64, MIXED = 0, 1


class MpsParams(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("quasi_compressibility_on", C.c_int32),
        ("higher_order_on", C.c_int32),
        ("pad0", C.c_int32),
        ("particle_distance", C.c_double),
        ("dt", C.c_double),
        ("domain_min", C.c_double * 3),
        ("domain_max", C.c_double * 3),
        ("density", C.c_double),
        ("kinematic_viscosity", C.c_double),
        ("gravity", C.c_double * 3),
        ("re_pressure", C.c_double),
        ("re_viscosity", C.c_double),
        ("re_surface", C.c_double),
        ("surface_threshold", C.c_double),
        ("compressibility", C.c_double),
        ("higher_order_gamma", C.c_double),
        ("relaxation", C.c_double),
        ("collision_distance", C.c_double),
        ("restitution", C.c_double),
        ("cfl", C.c_double),
    ]


class MpsStepStats(C.Structure):
    _fields_ = [
        ("courant", C.c_double),
        ("cg_relative_residual", C.c_double),
        ("cg_iterations", C.c_int64),
        ("refinements", C.c_int32),
        ("debug_log_count", C.c_int32),
        ("n_collision_candidates", C.c_int32),
        ("n_new_ghosts", C.c_int32),
        ("n_unconnected", C.c_int32),
        ("n_inner", C.c_int32),
        ("n_surface", C.c_int32),
        ("status", C.c_int32),
        ("ms_step", C.c_float),
        ("ms_solve", C.c_float),
        ("kernel_launches", C.c_int32),
        ("nnz_offdiag", C.c_int64),
        ("max_neighbors", C.c_int32),
    ]


class MpsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"mps error {code}: {msg}")
        self.code = code


_lib = None


def library_path() -> str:
    return _build.ENGINE_SO


def load(build_if_missing: bool = False):
    """Loads libmps_gb300.so (builds it first only if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise MpsError(MPS_ERR_NO_DEVICE,
                           f"{path} is missing: build it with `python -m mps_gb300.build`")
        _build.build_engine()
    L = C.CDLL(path)
    P = C.POINTER
    vp = C.c_void_p
    L.mps_create.argtypes = [P(MpsParams), C.c_int32, vp, vp, vp, P(vp)]
    L.mps_destroy.argtypes = [vp]
    L.mps_set_solver.argtypes = [vp, C.c_int32, C.c_double, C.c_int64]
    L.mps_set_multigrid.argtypes = [vp, C.c_int32, C.c_float, C.c_float]
    L.mps_set_multigrid.restype = C.c_int
    L.mps_step.argtypes = [vp, C.c_int32, P(MpsStepStats)]
    L.mps_run.argtypes = [vp, C.c_int32, P(MpsStepStats)]
    L.mps_download.argtypes = [vp] + [vp] * 8
    L.mps_upload.argtypes = [vp, vp, vp, vp]
    L.mps_particle_count.argtypes = [vp]
    L.mps_particle_count.restype = C.c_int32
    L.mps_stream.argtypes = [vp]
    L.mps_stream.restype = C.c_void_p
    L.mps_neighbors.argtypes = [vp, vp, vp, vp, P(C.c_int64)]
    L.mps_system.argtypes = [vp, vp, vp, vp, vp, P(C.c_int64)]
    L.mps_collisions.argtypes = [vp, vp, vp, vp, P(C.c_int32)]
    L.mps_last_error.restype = C.c_char_p
    for name in ("mps_create", "mps_destroy", "mps_set_solver", "mps_step", "mps_run",
                 "mps_download", "mps_upload", "mps_neighbors", "mps_system", "mps_collisions"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _check(rc):
    if rc != MPS_OK:
        raise MpsError(rc, _lib.mps_last_error().decode())


def make_params(p: dict) -> MpsParams:
    o = MpsParams()
    for name, _ in MpsParams._fields_:
        if name == "pad0" or name not in p:
            continue
        v = p[name]
        if name in ("domain_min", "domain_max", "gravity"):
            getattr(o, name)[:] = [float(x) for x in v]
        elif name in ("dim", "quasi_compressibility_on", "higher_order_on"):
            setattr(o, name, int(v))
        else:
            setattr(o, name, float(v))
    return o


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Engine:
    """One MPS scene on the current CUDA device (see include/mps_gb300.h)."""

    def __init__(self, params: dict, pos, vel, types, precision=FP64, tol=0.0, max_iter=0):
        L = load()
        self.n = int(len(types))
        self._prm = make_params(params)
        pos = np.ascontiguousarray(pos, np.float64).reshape(self.n, 3)
        vel = np.ascontiguousarray(vel, np.float64).reshape(self.n, 3)
        types = np.ascontiguousarray(types, np.int32)
        h = C.c_void_p()
        _check(L.mps_create(C.byref(self._prm), self.n, _p(pos), _p(vel), _p(types), C.byref(h)))
        self.h = h
        self.set_solver(precision, tol, max_iter)

    def close(self):
        if getattr(self, "h", None):
            _lib.mps_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stream_ptr(self) -> int:
        """cudaStream_t the engine launches on (for events around its work)."""
        return int(_lib.mps_stream(self.h) or 0)

    def set_solver(self, precision=FP64, tol=0.0, max_iter=0):
        _check(_lib.mps_set_solver(self.h, int(precision), float(tol), int(max_iter)))

    def set_multigrid(self, enabled=True, omega=0.9, scale=1.5):
        """Preconditioner of the MIXED solver: aggregation multigrid or Jacobi."""
        _check(_lib.mps_set_multigrid(self.h, 1 if enabled else 0, float(omega), float(scale)))

    @staticmethod
    def _stats(st: MpsStepStats) -> dict:
        return {k: getattr(st, k) for k, _ in MpsStepStats._fields_}

    def step(self, export=False) -> dict:
        st = MpsStepStats()
        _check(_lib.mps_step(self.h, 1 if export else 0, C.byref(st)))
        return self._stats(st)

    def run(self, n_steps: int) -> dict:
        st = MpsStepStats()
        _check(_lib.mps_run(self.h, int(n_steps), C.byref(st)))
        return self._stats(st)

    def state(self) -> dict:
        n = self.n
        d = dict(pos=np.zeros((n, 3)), vel=np.zeros((n, 3)), pressure=np.zeros(n),
                 min_pressure=np.zeros(n), ndr=np.zeros(n), type=np.zeros(n, np.int32),
                 bc=np.zeros(n, np.int32), dirichlet=np.zeros(n, np.int32))
        _check(_lib.mps_download(self.h, *[_p(d[k]) for k in (
            "pos", "vel", "pressure", "min_pressure", "ndr", "type", "bc", "dirichlet")]))
        return d

    def download_into(self, pos=None, vel=None, pressure=None, ndr=None, types=None, bc=None):
        _check(_lib.mps_download(self.h, _p(pos), _p(vel), _p(pressure), None, _p(ndr),
                                 _p(types), _p(bc), None))

    def upload(self, pos=None, vel=None, types=None):
        _check(_lib.mps_upload(self.h, _p(pos), _p(vel), _p(types)))

    def neighbors(self):
        tot = C.c_int64()
        _check(_lib.mps_neighbors(self.h, None, None, None, C.byref(tot)))
        off = np.zeros(self.n + 1, np.int64)
        ids = np.zeros(tot.value, np.int32)
        dist = np.zeros(tot.value)
        _check(_lib.mps_neighbors(self.h, _p(off), _p(ids), _p(dist), C.byref(tot)))
        return off, ids, dist

    def system(self):
        nnz = C.c_int64()
        src = np.zeros(self.n)
        _check(_lib.mps_system(self.h, _p(src), None, None, None, C.byref(nnz)))
        rp = np.zeros(self.n + 1, np.int64)
        col = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value)
        _check(_lib.mps_system(self.h, _p(src), _p(rp), _p(col), _p(val), C.byref(nnz)))
        return src, rp, col, val

    def collisions(self):
        cnt = C.c_int32()
        _check(_lib.mps_collisions(self.h, None, None, None, C.byref(cnt)))
        a = np.zeros(cnt.value, np.int32)
        b = np.zeros(cnt.value, np.int32)
        d = np.zeros(cnt.value)
        if cnt.value:
            _check(_lib.mps_collisions(self.h, _p(a), _p(b), _p(d), C.byref(cnt)))
        return a, b, d
