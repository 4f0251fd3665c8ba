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
 MPS_ERR_NONFINITE, MPS_ERR_NOT_CONVERGED, MPS_ERR_ASYMMETRIC) = range(9)
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
        ("graph_replayed", C.c_int32),
        ("solve_bytes", C.c_double),
    ]


class MpsSnapshot(C.Structure):
    """mps_snapshot (include/mps_gb300.h): an export snapshot in id order."""
    _fields_ = [
        ("n", C.c_int32),
        ("pos", C.POINTER(C.c_double)),
        ("vel", C.POINTER(C.c_double)),
        ("pressure", C.POINTER(C.c_double)),
        ("ndr", C.POINTER(C.c_double)),
        ("type", C.POINTER(C.c_int32)),
        ("bc", C.POINTER(C.c_int32)),
    ]


class MpsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"mps error {code}: {msg}")
        self.code = code


_lib = None


def library_path() -> str:
    """The engine library: MPS_GB300_LIB if set (an alternative build), else
    the in-tree build."""
    return os.environ.get("MPS_GB300_LIB") or _build.ENGINE_SO


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
    L.mps_set_initial_guess.argtypes = [vp, C.c_int32]
    L.mps_set_initial_guess.restype = C.c_int
    L.mps_set_collisions.argtypes = [vp, C.c_int32]
    L.mps_set_collisions.restype = C.c_int
    L.mps_set_graphs.argtypes = [vp, C.c_int32]
    L.mps_set_graphs.restype = C.c_int
    L.mps_step.argtypes = [vp, C.c_int32, P(MpsStepStats)]
    L.mps_run.argtypes = [vp, C.c_int32, P(MpsStepStats)]
    L.mps_run_report.argtypes = [vp, C.c_int32, vp]
    L.mps_run_report.restype = C.c_int
    L.mps_download.argtypes = [vp] + [vp] * 8
    L.mps_upload.argtypes = [vp, vp, vp, vp]
    L.mps_particle_count.argtypes = [vp]
    L.mps_particle_count.restype = C.c_int32
    L.mps_stream.argtypes = [vp]
    L.mps_stream.restype = C.c_void_p
    L.mps_neighbors.argtypes = [vp, vp, vp, vp, P(C.c_int64)]
    L.mps_system.argtypes = [vp, vp, vp, vp, vp, P(C.c_int64)]
    L.mps_collisions.argtypes = [vp, vp, vp, vp, P(C.c_int32)]
    L.mps_trajectory_create.argtypes = [vp, C.c_int32, C.c_int32, vp, C.c_int32, P(vp)]
    L.mps_trajectory_destroy.argtypes = [vp]
    L.mps_trajectory_forward.argtypes = [vp, vp, vp, vp, vp, vp]
    L.mps_trajectory_backward.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    for name in ("mps_trajectory_create", "mps_trajectory_destroy", "mps_trajectory_forward",
                 "mps_trajectory_backward"):
        getattr(L, name).restype = C.c_int
    L.mps_batch_create.argtypes = [C.c_int32, P(MpsParams), vp, vp, vp, vp, P(vp)]
    L.mps_batch_destroy.argtypes = [vp]
    L.mps_batch_set_solver.argtypes = [vp, C.c_double, C.c_int64]
    L.mps_batch_set_launch.argtypes = [vp, C.c_int32, C.c_double]
    L.mps_batch_launch_info.argtypes = [vp, P(C.c_int32), P(C.c_double), P(C.c_int32), vp,
                                        P(C.c_int32)]
    L.mps_batch_group_blocks.argtypes = [vp, vp]
    L.mps_batch_step.argtypes = [vp, C.c_int32, P(MpsStepStats), P(C.c_float)]
    L.mps_batch_size.argtypes = [vp]
    L.mps_batch_size.restype = C.c_int32
    L.mps_batch_scene.argtypes = [vp, C.c_int32]
    L.mps_batch_scene.restype = C.c_void_p
    L.mps_batch_stream.argtypes = [vp]
    L.mps_batch_stream.restype = C.c_void_p
    for name in ("mps_batch_create", "mps_batch_destroy", "mps_batch_set_solver",
                 "mps_batch_set_launch", "mps_batch_launch_info", "mps_batch_group_blocks",
                 "mps_batch_step"):
        getattr(L, name).restype = C.c_int
    L.mps_export_begin.argtypes = [vp]
    L.mps_export_view.argtypes = [vp, P(MpsSnapshot)]
    L.mps_export_write.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_double]
    L.mps_write_snapshot.argtypes = [P(MpsSnapshot), C.c_char_p, C.c_char_p, C.c_double]
    for name in ("mps_export_begin", "mps_export_view", "mps_export_write", "mps_write_snapshot"):
        getattr(L, name).restype = C.c_int
    L.mps_read_csv.argtypes = [C.c_char_p, C.c_int32, P(C.c_int32), P(C.c_double), vp, vp, vp]
    L.mps_read_csv.restype = C.c_int
    L.mps_selftest_wait_limit.argtypes = [P(C.c_int32), P(C.c_double)]
    L.mps_selftest_wait_limit.restype = C.c_int
    L.mps_check_symmetry.argtypes = [C.c_int32, vp, vp, vp, P(C.c_int32), P(C.c_int32)]
    L.mps_check_symmetry.restype = C.c_int
    L.mps_selftest_exact64.argtypes = [C.c_uint64, C.c_uint64, P(C.c_uint64)]
    L.mps_selftest_exact64.restype = C.c_int
    L.mps_last_error.restype = C.c_char_p
    for name in ("mps_create", "mps_destroy", "mps_set_solver", "mps_step", "mps_run",
                 "mps_download", "mps_upload", "mps_neighbors", "mps_system", "mps_collisions"):
        getattr(L, name).restype = C.c_int
    _lib = L
    return L


def _check(rc):
    if rc != MPS_OK:
        raise MpsError(rc, _lib.mps_last_error().decode())


def write_snapshot(snap: dict, csv_path=None, vtu_path=None, time=0.0):
    """The engine's CSV / VTU writers on host arrays (pos, vel: n x 3; pressure,
    ndr: n; type, bc: n int32), without an engine or a device."""
    L = load()
    n = len(snap["type"])
    keep = [np.ascontiguousarray(snap[k], dtype=np.float64) for k in ("pos", "vel", "pressure", "ndr")]
    keep += [np.ascontiguousarray(snap[k], dtype=np.int32) for k in ("type", "bc")]
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
    s = MpsSnapshot(n, dp(keep[0]), dp(keep[1]), dp(keep[2]), dp(keep[3]), ip(keep[4]), ip(keep[5]))
    enc = lambda q: None if q is None else os.fsencode(q)
    _check(L.mps_write_snapshot(C.byref(s), enc(csv_path), enc(vtu_path), float(time)))


def read_particles_csv(path):
    """The engine's particle CSV reader (the reference's importInitialCondition
    format): (time, pos n x 3, vel n x 3, type n int32).  Host only."""
    L = load()
    n = C.c_int32(0)
    tm = C.c_double(0.0)
    enc = os.fsencode(path)
    rc = L.mps_read_csv(enc, 0, C.byref(n), C.byref(tm), None, None, None)
    if rc not in (0, 3):
        _check(rc)
    pos = np.zeros((n.value, 3))
    vel = np.zeros((n.value, 3))
    typ = np.zeros(n.value, np.int32)
    _check(L.mps_read_csv(enc, n.value, C.byref(n), C.byref(tm), _p(pos), _p(vel), _p(typ)))
    return tm.value, pos, vel, typ


def selftest_wait_limit():
    """Runs the device-side wait-limit self-test (include/mps_gb300.h):
    (return code, blocks that gave up, seconds)."""
    L = load()
    g = C.c_int32(0)
    sec = C.c_double(0.0)
    rc = L.mps_selftest_wait_limit(C.byref(g), C.byref(sec))
    return rc, g.value, sec.value


def check_symmetry(row_ptr, col, val):
    """mps_check_symmetry on a CSR matrix: (return code, i, j, message); i, j
    are the first asymmetric pair (-1, -1 when symmetric)."""
    L = load()
    rp = np.ascontiguousarray(row_ptr, np.int64)
    cl = np.ascontiguousarray(col, np.int32)
    vl = np.ascontiguousarray(val, np.float64)
    i, j = C.c_int32(-2), C.c_int32(-2)
    rc = L.mps_check_symmetry(len(rp) - 1, _p(rp), _p(cl), _p(vl), C.byref(i), C.byref(j))
    return rc, i.value, j.value, (L.mps_last_error().decode() if rc else "")


def selftest_exact64(n: int, seed: int = 1):
    """mps_selftest_exact64: the integer-pipe FP64 square root and division
    against the GPU's FP64 instructions on n seeded cases of each.  Returns
    (return code, dict with sqrt_mismatches, div_mismatches, sqrt_fast,
    div_fast, first_bad, other_mismatches)."""
    L = load()
    res = (C.c_uint64 * 8)()
    rc = L.mps_selftest_exact64(int(n), int(seed), res)
    return rc, {"sqrt_mismatches": res[0], "div_mismatches": res[1], "sqrt_fast": res[2],
                "div_fast": res[3], "first_bad": (res[4], res[5], res[6]), "other_mismatches": res[7]}


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

    @classmethod
    def borrowed(cls, handle, n: int) -> "Engine":
        """A view of an engine owned elsewhere (a batch's scene): not destroyed here."""
        e = cls.__new__(cls)
        e.n = int(n)
        e.h = None
        e._borrowed = C.c_void_p(handle)
        return e

    @property
    def _h(self):
        return self.h if self.h is not None else getattr(self, "_borrowed", None)

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
        return int(_lib.mps_stream(self._h) or 0)

    def set_solver(self, precision=FP64, tol=0.0, max_iter=0):
        _check(_lib.mps_set_solver(self._h, int(precision), float(tol), int(max_iter)))

    MG_JACOBI, MG_ADDITIVE, MG_MULTIPLICATIVE, MG_SMOOTHED = 0, 1, 2, 3

    def set_multigrid(self, mode=1, omega=0.0, scale=0.0):
        """Preconditioner of the MIXED solver: 0 Jacobi, 1 multigrid additive at
        the particle level (default), 2 multiplicative V(1,1), 3 additive with
        the smoothed particle-to-cell transfer, 4 mode 1's preconditioner with the
        operator applied after the cycle (True/False map to 1/0).
        omega/scale 0 take the mode's default weights."""
        mode = int(mode) if not isinstance(mode, bool) else (1 if mode else 0)
        _check(_lib.mps_set_multigrid(self._h, mode, float(omega), float(scale)))

    def set_initial_guess(self, previous=True):
        """MIXED solver's initial guess: the previous step's solution of the same
        particles (default) or zero (the reference's CG start)."""
        _check(_lib.mps_set_initial_guess(self._h, 1 if previous else 0))

    def set_collisions(self, serial=False):
        """Collision pairs applied in parallel (default) or by one thread in order."""
        _check(_lib.mps_set_collisions(self._h, 1 if serial else 0))

    def set_graphs(self, enabled=True):
        """Non-export steps as CUDA graph replays (default) or eager launches."""
        _check(_lib.mps_set_graphs(self._h, 1 if enabled else 0))

    @staticmethod
    def _stats(st: MpsStepStats) -> dict:
        return {k: getattr(st, k) for k, _ in MpsStepStats._fields_}

    def step(self, export=False) -> dict:
        st = MpsStepStats()
        _check(_lib.mps_step(self._h, 1 if export else 0, C.byref(st)))
        return self._stats(st)

    def run(self, n_steps: int) -> dict:
        st = MpsStepStats()
        _check(_lib.mps_run(self._h, int(n_steps), C.byref(st)))
        return self._stats(st)

    def run_report(self, n_steps: int) -> list:
        """n non-export steps with one host wait per up to 256 steps; the
        stats of every step (mps_run_report)."""
        st = (MpsStepStats * max(int(n_steps), 1))()
        _check(_lib.mps_run_report(self._h, int(n_steps), st))
        return [self._stats(s) for s in st[:int(n_steps)]]

    def state(self) -> dict:
        n = self.n
        d = dict(pos=np.zeros((n, 3)), vel=np.zeros((n, 3)), pressure=np.zeros(n),
                 min_pressure=np.zeros(n), ndr=np.zeros(n), type=np.zeros(n, np.int32),
                 bc=np.zeros(n, np.int32), dirichlet=np.zeros(n, np.int32))
        _check(_lib.mps_download(self._h, *[_p(d[k]) for k in (
            "pos", "vel", "pressure", "min_pressure", "ndr", "type", "bc", "dirichlet")]))
        return d

    def download_into(self, pos=None, vel=None, pressure=None, ndr=None, types=None, bc=None):
        _check(_lib.mps_download(self._h, _p(pos), _p(vel), _p(pressure), None, _p(ndr),
                                 _p(types), _p(bc), None))

    def export_begin(self):
        """Snapshot the state for export; the following steps may run at once."""
        _check(_lib.mps_export_begin(self._h))

    def export_snapshot(self) -> dict:
        """Waits for the snapshot of the last export_begin; copies of its arrays."""
        s = MpsSnapshot()
        _check(_lib.mps_export_view(self._h, C.byref(s)))
        n = s.n
        arr = lambda p, k: np.ctypeslib.as_array(p, shape=(k,)).copy()
        return dict(pos=arr(s.pos, 3 * n).reshape(n, 3), vel=arr(s.vel, 3 * n).reshape(n, 3),
                    pressure=arr(s.pressure, n), ndr=arr(s.ndr, n), type=arr(s.type, n),
                    bc=arr(s.bc, n))

    def export_write(self, csv_path=None, vtu_path=None, time=0.0):
        """Waits for the snapshot and writes the reference's CSV / VTU files
        (releases the GIL: may run on a writer thread while steps go on)."""
        enc = lambda p: None if p is None else os.fsencode(p)
        _check(_lib.mps_export_write(self._h, enc(csv_path), enc(vtu_path), float(time)))

    def upload(self, pos=None, vel=None, types=None):
        _check(_lib.mps_upload(self._h, _p(pos), _p(vel), _p(types)))

    def neighbors(self):
        tot = C.c_int64()
        _check(_lib.mps_neighbors(self._h, None, None, None, C.byref(tot)))
        off = np.zeros(self.n + 1, np.int64)
        ids = np.zeros(tot.value, np.int32)
        dist = np.zeros(tot.value)
        _check(_lib.mps_neighbors(self._h, _p(off), _p(ids), _p(dist), C.byref(tot)))
        return off, ids, dist

    def system(self):
        nnz = C.c_int64()
        src = np.zeros(self.n)
        _check(_lib.mps_system(self._h, _p(src), None, None, None, C.byref(nnz)))
        rp = np.zeros(self.n + 1, np.int64)
        col = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value)
        _check(_lib.mps_system(self._h, _p(src), _p(rp), _p(col), _p(val), C.byref(nnz)))
        return src, rp, col, val

    def collisions(self):
        cnt = C.c_int32()
        _check(_lib.mps_collisions(self._h, None, None, None, C.byref(cnt)))
        a = np.zeros(cnt.value, np.int32)
        b = np.zeros(cnt.value, np.int32)
        d = np.zeros(cnt.value)
        if cnt.value:
            _check(_lib.mps_collisions(self._h, _p(a), _p(b), _p(d), C.byref(cnt)))
        return a, b, d


class Trajectory:
    """n_steps of an engine from its current state, with the adjoint of the
    whole step (include/mps_gb300.h, mps_trajectory_*).  Arrays are numpy,
    particle-id order, shape (n, 3) for vectors."""

    def __init__(self, engine: Engine, n_steps: int, checkpoint_every: int = 20, sensors=()):
        self.engine = engine
        self.n = engine.n
        self.steps = int(n_steps)
        self.sensors = np.ascontiguousarray(sensors, np.int32)
        h = C.c_void_p()
        _check(_lib.mps_trajectory_create(engine._h, self.steps, int(checkpoint_every),
                                          _p(self.sensors) if len(self.sensors) else None,
                                          len(self.sensors), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            _lib.mps_trajectory_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, vel0=None, gravity=None):
        """-> (sensor pressure [steps, n_sensors], final positions, final velocities)."""
        v0 = None if vel0 is None else np.ascontiguousarray(vel0, np.float64).reshape(self.n, 3)
        g = None if gravity is None else np.ascontiguousarray(gravity, np.float64).reshape(3)
        sp = np.zeros((self.steps, len(self.sensors)))
        pos = np.zeros((self.n, 3))
        vel = np.zeros((self.n, 3))
        _check(_lib.mps_trajectory_forward(self.h, _p(v0), _p(g), _p(sp) if sp.size else None,
                                           _p(pos), _p(vel)))
        return sp, pos, vel

    def backward(self, d_sensor=None, d_pos=None, d_vel=None):
        """Vector-Jacobian product of the last forward -> (dL/dpos0, dL/dvel0, dL/dgravity)."""
        def arr(a, shape):
            return None if a is None else np.ascontiguousarray(a, np.float64).reshape(shape)
        ds = arr(d_sensor, (self.steps, len(self.sensors)))
        dp, dv = arr(d_pos, (self.n, 3)), arr(d_vel, (self.n, 3))
        gp, gv, gg = np.zeros((self.n, 3)), np.zeros((self.n, 3)), np.zeros(3)
        _check(_lib.mps_trajectory_backward(self.h, _p(ds) if ds is not None and ds.size else None,
                                            _p(dp), _p(dv), _p(gp), _p(gv), _p(gg)))
        return gp, gv, gg


class Batch:
    """Many independent scenes advanced together with one shared solve launch
    per step (include/mps_gb300.h, mps_batch_*)."""

    def __init__(self, scenes, tol=1e-8, max_iter=0):
        """scenes: list of (params, pos[n,3], vel[n,3], types[n])."""
        L = load()
        self.counts = np.array([len(s[3]) for s in scenes], np.int32)
        prms = (MpsParams * len(scenes))(*[make_params(s[0]) for s in scenes])
        pos = np.ascontiguousarray(np.concatenate([np.asarray(s[1], np.float64).reshape(-1, 3)
                                                   for s in scenes]))
        vel = np.ascontiguousarray(np.concatenate([np.asarray(s[2], np.float64).reshape(-1, 3)
                                                   for s in scenes]))
        typ = np.ascontiguousarray(np.concatenate([np.asarray(s[3], np.int32) for s in scenes]))
        h = C.c_void_p()
        _check(L.mps_batch_create(len(scenes), prms, _p(self.counts), _p(pos), _p(vel), _p(typ),
                                  C.byref(h)))
        self.h = h
        self.set_solver(tol, max_iter)

    def close(self):
        if getattr(self, "h", None):
            _lib.mps_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.counts)

    def set_solver(self, tol=1e-8, max_iter=0):
        _check(_lib.mps_batch_set_solver(self.h, float(tol), int(max_iter)))

    def set_launch(self, block=0, alpha=1.0):
        """block 0: autotune at the next step; else 256/512/1024 threads and alpha."""
        _check(_lib.mps_batch_set_launch(self.h, int(block), float(alpha)))

    def launch_info(self) -> dict:
        blk, al, grid, nt = C.c_int32(), C.c_double(), C.c_int32(), C.c_int32()
        ms = np.zeros(16, np.float32)
        _check(_lib.mps_batch_launch_info(self.h, C.byref(blk), C.byref(al), C.byref(grid),
                                          _p(ms), C.byref(nt)))
        gb = np.zeros(len(self), np.int32)
        if blk.value:
            _check(_lib.mps_batch_group_blocks(self.h, _p(gb)))
        return {"block": blk.value, "alpha": al.value, "grid": grid.value,
                "tune_ms": ms[:nt.value].tolist(), "group_blocks": gb.tolist()}

    def step(self, n_steps=1):
        """-> (list of per-scene stats dicts of the last step, batch step ms)."""
        st = (MpsStepStats * len(self))()
        ms = C.c_float()
        _check(_lib.mps_batch_step(self.h, int(n_steps), st, C.byref(ms)))
        return [Engine._stats(s) for s in st], ms.value

    def stream_ptr(self) -> int:
        return int(_lib.mps_batch_stream(self.h) or 0)

    def scene(self, s: int) -> Engine:
        """Borrowed engine view of scene s (state(), neighbors(), ...)."""
        return Engine.borrowed(_lib.mps_batch_scene(self.h, int(s)), int(self.counts[s]))
