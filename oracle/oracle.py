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
        ip = C.POINTER(C.c_int)
        lib.oracle_lensing_lrange.restype = None
        lib.oracle_lensing_lrange.argtypes = [ip, C.c_int, C.c_int, C.c_int, C.c_double, ip]
        lib.oracle_interpolate_cls.restype = None
        lib.oracle_interpolate_cls.argtypes = [ip, C.c_int, dp, dp, C.c_double, dp]
        lib.oracle_lens_cls_apodized.restype = C.c_int
        lib.oracle_lens_cls_apodized.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, dp, dp]
        lib.oracle_mode_setup.restype = C.c_int
        lib.oracle_mode_setup.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_int), dp]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _view(tables):
    """A Tables handle's view, or a CambGpuTables view itself (the transfer half)."""
    return tables.view if hasattr(tables, "view") else tables


def evolve_sources(tables, nthreads=0, k_range=None, with_evals=False):
    v = _view(tables)
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


def load_template():
    """The high-L template table [8001][4] (TT, EE, TE, PP by l) shipped with the package."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "camb_gb300", "data", "highl_template.f64")
    return np.fromfile(path, dtype="<f8").reshape(8001, 4)


def interpolate_cls(ls, icl, scale, tmpl=None):
    """InterpolateCls: icl [nl][6] at the sampled ls -> [ls[-1]+1][6] at every l."""
    tmpl = load_template() if tmpl is None else tmpl
    ls = np.ascontiguousarray(ls, dtype=np.int32)
    icl = np.ascontiguousarray(icl, dtype=np.float64)
    out = np.zeros((int(ls[-1]) + 1, 6))
    load().oracle_interpolate_cls(ls.ctypes.data_as(C.POINTER(C.c_int)), len(ls), _dp(icl), _dp(tmpl), scale,
                                  _dp(out))
    return out


def lensing_lrange(ls, max_l, lens_output_margin=200, lens_accuracy_boost=1.0):
    ls = np.ascontiguousarray(ls, dtype=np.int32)
    out = (C.c_int * 2)()
    load().oracle_lensing_lrange(ls.ctypes.data_as(C.POINTER(C.c_int)), len(ls), max_l, lens_output_margin,
                                 lens_accuracy_boost, out)
    return out[0], out[1]


def lens_cls(all_cls, ls, max_l, lmin=2, lens_output_margin=200, lens_accuracy_boost=1.0, tmpl=None):
    """CorrFuncFullSkyApodized: all_cls [max_l+1][>=4] holding TT EE TE and the C_Phi
    column of InterpolateCls -> lensed [lmax_lensed+1][4] TT EE BB TE."""
    tmpl = load_template() if tmpl is None else tmpl
    lmax, lmax_lensed = lensing_lrange(ls, max_l, lens_output_margin, lens_accuracy_boost)
    cl = np.ascontiguousarray(all_cls[: max_l + 1, :4], dtype=np.float64)
    out = np.zeros((lmax_lensed + 1, 4))
    rc = load().oracle_lens_cls_apodized(_dp(cl), max_l, lmin, lmax, lmax_lensed, lens_output_margin,
                                         lens_accuracy_boost, _dp(tmpl), _dp(out))
    if rc:
        raise RuntimeError("lensing amplitude check failed")
    return out


def evolve_transfer(tables, nthreads=0, with_evals=False):
    """GetTransfer for every transfer k: [ntimes][nk][13] float32 (TransferData order)."""
    v = _view(tables)
    lib = load()
    lib.oracle_evolve_transfer.restype = C.c_int
    lib.oracle_evolve_transfer.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_long)]
    out = np.zeros((v.num_transfer_times, v.nk, 13), dtype=np.float32)
    evals = np.zeros(v.nk, dtype=np.int64)
    rc = lib.oracle_evolve_transfer(C.addressof(v), out.ctypes.data_as(C.POINTER(C.c_float)), nthreads,
                                    evals.ctypes.data_as(C.POINTER(C.c_long)))
    if rc:
        raise RuntimeError(f"oracle transfer evolution failed: {rc}")
    return (out, evals) if with_evals else out


def evolve_combined(tables, nthreads=0):
    """The reference's run that wants the CMB and transfer functions (CalcScalarSources with
    the transfer stops, then TransferOut above the source grid): (LinearSrc [ntau][nsrc][nk]
    of the CMB view, TransferData [ntimes][nk_transfer][13] of the transfer half)."""
    v, t = tables.view, tables.transfer_view()
    lib = load()
    lib.oracle_evolve_combined.restype = C.c_int
    lib.oracle_evolve_combined.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_float),
                                           C.c_int]
    src = np.zeros((v.ntau, v.nsrc, v.nk))
    tr = np.zeros((t.num_transfer_times, t.nk, 13), dtype=np.float32)
    rc = lib.oracle_evolve_combined(C.addressof(v), C.addressof(t), _dp(src), tr.ctypes.data_as(C.POINTER(C.c_float)),
                                    nthreads)
    if rc:
        raise RuntimeError(f"oracle combined evolution failed: {rc}")
    return src, tr


def sigma8(tables, tr):
    """Transfer_Get_sigmas at R = 8 Mpc/h: (sigma8, sigma2_vdelta_8) per transfer time."""
    v = _view(tables)
    lib = load()
    lib.oracle_sigma8.restype = None
    lib.oracle_sigma8.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
    tr = np.ascontiguousarray(tr, dtype=np.float32)
    s8 = np.zeros(v.num_transfer_times)
    sv = np.zeros(v.num_transfer_times)
    lib.oracle_sigma8(C.addressof(v), tr.ctypes.data_as(C.POINTER(C.c_float)), _dp(s8), _dp(sv))
    return s8, sv
