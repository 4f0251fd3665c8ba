"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.  The oracle is a
restatement of the reference's hot path (iori3150/MPS src/mps.cpp and
src/bucket.cpp); see mps_oracle.h for what pins it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


class OrcParams(C.Structure):
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


class OrcStats(C.Structure):
    _fields_ = [
        ("courant", C.c_double),
        ("cg_iterations", C.c_int64),
        ("cg_error", C.c_double),
        ("debug_log_count", C.c_int32),
        ("n_collision_candidates", C.c_int32),
        ("n_inner", C.c_int32),
        ("n_surface", C.c_int32),
    ]


def build():
    """Compile liboracle.so from its C++ source (plain g++, no GPU)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.POINTER
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [P(OrcParams), C.c_int32, P(C.c_double), P(C.c_double), P(C.c_int32)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_cg.argtypes = [C.c_void_p, C.c_double, C.c_int64, C.c_int32]
        L.orc_step.argtypes = [C.c_void_p, C.c_int32, P(OrcStats)]
        L.orc_get_state.argtypes = [C.c_void_p] + [C.c_void_p] * 8
        L.orc_neighbor_total.restype = C.c_int64
        L.orc_neighbor_total.argtypes = [C.c_void_p]
        L.orc_get_neighbors.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_matrix_nnz.restype = C.c_int64
        L.orc_matrix_nnz.argtypes = [C.c_void_p]
        L.orc_get_system.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.orc_collision_count.restype = C.c_int32
        L.orc_collision_count.argtypes = [C.c_void_p]
        L.orc_get_collisions.argtypes = [C.c_void_p] + [C.c_void_p] * 3
        L.orc_ref_values.argtypes = [C.c_int32, C.c_double, C.c_double, P(C.c_double), P(C.c_double)]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def make_params(p: dict) -> OrcParams:
    o = OrcParams()
    for name, _ in OrcParams._fields_:
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


def ref_values(dim, l0, re):
    n0, lam = C.c_double(), C.c_double()
    lib().orc_ref_values(int(dim), float(l0), float(re), C.byref(n0), C.byref(lam))
    return n0.value, lam.value


class Oracle:
    """One reference-equivalent MPS instance on the CPU."""

    def __init__(self, params: dict, pos, vel, types):
        self.n = int(len(types))
        self._prm = make_params(params)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(self.n, 3)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(self.n, 3)
        types = np.ascontiguousarray(types, dtype=np.int32)
        self.h = lib().orc_create(C.byref(self._prm), self.n,
                                  pos.ctypes.data_as(C.POINTER(C.c_double)),
                                  vel.ctypes.data_as(C.POINTER(C.c_double)),
                                  types.ctypes.data_as(C.POINTER(C.c_int32)))

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_cg(self, tol=np.finfo(np.float64).eps, max_iter=-1, solves=2):
        lib().orc_set_cg(self.h, float(tol), int(max_iter), int(solves))

    def step(self, export=False) -> dict:
        st = OrcStats()
        lib().orc_step(self.h, 1 if export else 0, C.byref(st))
        return {k: getattr(st, k) for k, _ in OrcStats._fields_}

    def state(self) -> dict:
        n = self.n
        d = dict(pos=np.zeros((n, 3)), vel=np.zeros((n, 3)), pressure=np.zeros(n),
                 min_pressure=np.zeros(n), ndr=np.zeros(n), type=np.zeros(n, np.int32),
                 bc=np.zeros(n, np.int32), dirichlet=np.zeros(n, np.int32))
        lib().orc_get_state(self.h, *[_ptr(d[k]) for k in
                                      ("pos", "vel", "pressure", "min_pressure", "ndr", "type", "bc",
                                       "dirichlet")])
        return d

    def neighbors(self):
        tot = lib().orc_neighbor_total(self.h)
        off = np.zeros(self.n + 1, np.int64)
        ids = np.zeros(tot, np.int32)
        dist = np.zeros(tot, np.float64)
        lib().orc_get_neighbors(self.h, _ptr(off), _ptr(ids), _ptr(dist))
        return off, ids, dist

    def system(self):
        nnz = lib().orc_matrix_nnz(self.h)
        src = np.zeros(self.n)
        rp = np.zeros(self.n + 1, np.int64)
        col = np.zeros(nnz, np.int32)
        val = np.zeros(nnz)
        lib().orc_get_system(self.h, _ptr(src), _ptr(rp), _ptr(col), _ptr(val))
        return src, rp, col, val

    def collisions(self):
        k = lib().orc_collision_count(self.h)
        a = np.zeros(k, np.int32)
        b = np.zeros(k, np.int32)
        d = np.zeros(k)
        if k:
            lib().orc_get_collisions(self.h, _ptr(a), _ptr(b), _ptr(d))
        return a, b, d
