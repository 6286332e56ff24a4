"""ctypes binding of the CPU oracle (oracle/build/liboracle.so).

Test infrastructure only: the oracle restates ompVC's algorithm on the CPU
and is used as the checker for the engine's results."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "build", "liboracle.so")
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None


def lib():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-s"], check=True, capture_output=True)
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int, C.c_int]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_cart.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int,
                                   C.c_double, C.c_double, C.c_int]
        L.orc_set_unstruct.argtypes = [C.c_void_p, C.c_int, _dp, C.c_int, _ip, _ip]
        L.orc_set_bounds.argtypes = [C.c_void_p, _dp]
        L.orc_set_frames.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_double]
        L.orc_set_integrator.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int]
        L.orc_set_rkf.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        L.orc_advect.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _ip, _ip, _dp, C.c_double, C.c_double,
                                 C.POINTER(C.c_longlong)]
        L.orc_velocity.argtypes = [C.c_void_p, C.c_int, _dp, _ip, _ip, C.c_double, _dp]
        L.orc_local_search.argtypes = [C.c_void_p, C.c_int, _dp, _ip, _ip]
        L.orc_global_search.argtypes = [C.c_void_p, C.c_int, _dp, _ip]
        L.orc_max_eig.restype = C.c_double
        L.orc_max_eig.argtypes = [_dp]
        L.orc_run.argtypes = [C.c_char_p, C.c_int, _dp, C.POINTER(C.c_longlong), C.c_char_p, C.c_int]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def _i(a):
    return a.ctypes.data_as(_ip) if a is not None else None


class Oracle:
    def __init__(self, dims, mesh_type):
        self.L = lib()
        self.h = self.L.orc_create(dims, mesh_type)
        assert self.h
        self._keep = []

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)

    def set_cart(self, *a):
        assert self.L.orc_set_cart(self.h, *a) == 0

    def set_unstruct(self, xyz, conn, adj):
        xyz = np.ascontiguousarray(xyz, np.float64)
        conn = np.ascontiguousarray(conn, np.int32)
        adj = np.ascontiguousarray(adj, np.int32)
        assert self.L.orc_set_unstruct(self.h, xyz.shape[0], _d(xyz), conn.shape[0], _i(conn), _i(adj)) == 0

    def set_bounds(self, b):
        b = np.ascontiguousarray(b, np.float64)
        assert self.L.orc_set_bounds(self.h, _d(b)) == 0

    def set_frames(self, f0, f1, tmin, tmax):
        f0 = np.ascontiguousarray(f0, np.float64)
        f1 = np.ascontiguousarray(f1, np.float64)
        self._keep = [f0, f1]
        assert self.L.orc_set_frames(self.h, _d(f0), _d(f1), tmin, tmax) == 0

    def set_integrator(self, t, h, ex=0):
        assert self.L.orc_set_integrator(self.h, t, h, ex) == 0

    def set_rkf(self, acc, hmin, hmax):
        assert self.L.orc_set_rkf(self.h, acc, hmin, hmax) == 0

    def advect(self, X, V, eid, left, ldt, t0, t1):
        steps = C.c_longlong(0)
        rc = self.L.orc_advect(self.h, X.shape[0], _d(X), _d(V), _i(eid), _i(left), _d(ldt), t0, t1, C.byref(steps))
        assert rc == 0, rc
        return steps.value

    def velocity(self, X, eid, left, tq):
        out = np.zeros_like(X)
        assert self.L.orc_velocity(self.h, X.shape[0], _d(X), _i(eid), _i(left), tq, _d(out)) == 0
        return out

    def local_search(self, X, guess):
        out = np.empty(X.shape[0], np.int32)
        assert self.L.orc_local_search(self.h, X.shape[0], _d(np.ascontiguousarray(X, np.float64)),
                                       _i(np.ascontiguousarray(guess, np.int32)), _i(out)) == 0
        return out

    def global_search(self, X):
        out = np.empty(X.shape[0], np.int32)
        assert self.L.orc_global_search(self.h, X.shape[0], _d(np.ascontiguousarray(X, np.float64)), _i(out)) == 0
        return out


def max_eig(a):
    a = np.ascontiguousarray(a, np.float64).reshape(9)
    return lib().orc_max_eig(_d(a))


def run(in_path, nthreads=0):
    secs = C.c_double(0)
    steps = C.c_longlong(0)
    err = C.create_string_buffer(1024)
    rc = lib().orc_run(in_path.encode(), nthreads, C.byref(secs), C.byref(steps), err, 1024)
    return rc, secs.value, steps.value, err.value.decode()
