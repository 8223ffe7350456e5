"""ORACLE -- test infrastructure only.

ctypes wrapper of liboracle.so, the CPU restatement of the reference's scalar flat
hot path.  Takes the same CambGpuTables view the GPU library consumes.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        lib.oracle_evolve_scalar_sources.restype = C.c_int
        lib.oracle_evolve_scalar_sources.argtypes = [C.c_void_p, dp, C.c_int, C.POINTER(C.c_long), C.c_int, C.c_int]
        lib.oracle_los_flat.restype = C.c_int
        lib.oracle_los_flat.argtypes = [C.c_void_p, dp, dp, C.c_int]
        lib.oracle_calc_scal_cls.restype = C.c_int
        lib.oracle_calc_scal_cls.argtypes = [C.c_void_p, dp, dp]
        lib.oracle_mode_setup.restype = C.c_int
        lib.oracle_mode_setup.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_int), dp]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def evolve_sources(tables, nthreads=0, k_range=None, with_evals=False):
    v = tables.view
    out = np.zeros((v.ntau, v.nsrc, v.nk))
    evals = np.zeros(v.nk, dtype=np.int64)
    lo, hi = k_range if k_range else (0, v.nk)
    rc = load().oracle_evolve_scalar_sources(C.addressof(v), _dp(out), nthreads,
                                             evals.ctypes.data_as(C.POINTER(C.c_long)), lo, hi)
    if rc:
        raise RuntimeError(f"oracle evolution failed: {rc}")
    return (out, evals) if with_evals else out


def los(tables, src, nthreads=0):
    v = tables.view
    src = np.ascontiguousarray(src, dtype=np.float64)
    out = np.zeros((v.nq, v.nl, v.nsrc))
    load().oracle_los_flat(C.addressof(v), _dp(src), _dp(out), nthreads)
    return out


def cls(tables, delta):
    v = tables.view
    delta = np.ascontiguousarray(delta, dtype=np.float64)
    out = np.zeros((v.nl, 6))
    load().oracle_calc_scal_cls(C.addressof(v), _dp(delta), _dp(out))
    return out


def mode_setup(tables, q):
    l3 = (C.c_int * 3)()
    ts = C.c_double()
    load().oracle_mode_setup(C.addressof(tables.view), q, l3, C.byref(ts))
    return (l3[0], l3[1], l3[2]), ts.value
