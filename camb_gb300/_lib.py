"""ctypes binding of libcambgpu.so (declarations in include/cambgpu.h).

This is the same kind of binding the reference's Python layer uses for its
compiled library (camb/baseconfig.py loads camblib.so through ctypes).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_c_double_p = C.POINTER(C.c_double)
_c_int_p = C.POINTER(C.c_int)


class CambGpuParams(C.Structure):
    _fields_ = [
        ("H0", C.c_double), ("ombh2", C.c_double), ("omch2", C.c_double), ("omk", C.c_double),
        ("TCMB", C.c_double), ("YHe", C.c_double),
        ("nnu", C.c_double),
        ("mnu", C.c_double),
        ("num_massive_neutrinos", C.c_int),
        ("optical_depth", C.c_double),
        ("reion_delta_redshift", C.c_double),
        ("As", C.c_double), ("ns", C.c_double), ("nrun", C.c_double), ("pivot_scalar", C.c_double),
        ("Alens", C.c_double),
        ("max_l", C.c_int),
        ("max_eta_k", C.c_double),
        ("do_lensing", C.c_int),
        ("AccuracyBoost", C.c_double), ("lAccuracyBoost", C.c_double), ("lSampleBoost", C.c_double),
        ("IntTolBoost", C.c_double), ("TimeStepBoost", C.c_double),
        ("SourcekAccuracyBoost", C.c_double), ("IntkAccuracyBoost", C.c_double), ("BesselBoost", C.c_double),
        ("BessIntBoost", C.c_double),
        ("TimeSwitchBoost", C.c_double), ("LimberBoost", C.c_double), ("BackgroundTimeStepBoost", C.c_double),
        ("accurate_polarization", C.c_int), ("accurate_reionization", C.c_int),
        ("LensingBoost", C.c_double),
        ("want_cls", C.c_int), ("want_transfer", C.c_int), ("transfer_high_precision", C.c_int),
        ("transfer_kmax", C.c_double), ("num_transfer_redshifts", C.c_int), ("transfer_redshifts", C.c_double * 256),
        ("reion_use_optical_depth", C.c_int), ("reion_redshift", C.c_double),
        ("recfast_no_rosenbrock", C.c_int),
    ]


class CambGpuModeSpec(C.Structure):
    _fields_ = [("q", C.c_double), ("taustart", C.c_double), ("tight_switch_tau", C.c_double),
                ("lmaxg", C.c_int), ("lmaxgpol", C.c_int), ("lmaxnr", C.c_int), ("lmaxnu", C.c_int),
                ("nq0", C.c_int * 3), ("pad", C.c_int),
                ("nu_l_boost", C.c_double * 3), ("nu_approx_time", C.c_double * 3)]


class CambGpuTables(C.Structure):
    _fields_ = [
        ("grhog", C.c_double), ("grhor", C.c_double), ("grhornomass", C.c_double), ("grhoc", C.c_double),
        ("grhob", C.c_double), ("grhov", C.c_double), ("grhok", C.c_double),
        ("adotrad", C.c_double), ("tau0", C.c_double), ("DMt0", C.c_double), ("taurst", C.c_double),
        ("taurend", C.c_double), ("tau_maxvis", C.c_double), ("matter_verydom_tau", C.c_double),
        ("akthom", C.c_double), ("fHe", C.c_double),
        ("nu_eig", C.c_int), ("nqmax", C.c_int),
        ("nu_masses", C.c_double * 3), ("grhormass", C.c_double * 3), ("nu_tau_nonrel", C.c_double * 3),
        ("nu_q", _c_double_p), ("nu_int_kernel", _c_double_p), ("nu_tau_notmassless", _c_double_p),
        ("nthermo", C.c_int),
        ("tauminn", C.c_double), ("dlntau", C.c_double), ("dlntau_inv", C.c_double), ("tight_tau", C.c_double),
        ("thermo_horner", _c_double_p), ("dotmu", _c_double_p), ("ddotmu", _c_double_p), ("cs2", _c_double_p),
        ("dddotmu", _c_double_p), ("ddddotmu", _c_double_p), ("emmu", _c_double_p), ("demmu", _c_double_p),
        ("ntau", C.c_int), ("tau_points", _c_double_p), ("tau_dpoints", _c_double_p),
        ("nk", C.c_int), ("q_evolve", _c_double_p), ("modes", C.POINTER(CambGpuModeSpec)),
        ("nq", C.c_int), ("q_int", _c_double_p), ("dq_int", _c_double_p),
        ("nl", C.c_int), ("ls", _c_int_p),
        ("num_xx", C.c_int), ("bess_x", _c_double_p), ("bessel_horner", _c_double_p),
        ("nsrc", C.c_int), ("want_late_time", C.c_int),
        ("max_etak_scalar", C.c_double), ("tol1", C.c_double), ("max_bessels_etak", C.c_double),
        ("AccuracyBoost", C.c_double), ("IntTolBoost", C.c_double), ("TimeSwitchBoost", C.c_double),
        ("BessIntBoost", C.c_double), ("LimberBoost", C.c_double),
        ("lAccuracyBoost", C.c_double),
        ("accurate_polarization", C.c_int), ("accurate_reionization", C.c_int),
        ("As", C.c_double), ("ns", C.c_double), ("nrun", C.c_double), ("pivot_scalar", C.c_double),
        ("Alens", C.c_double),
        ("max_l", C.c_int), ("do_lensing", C.c_int), ("cl_template_scale", C.c_double),
        ("lens_accuracy_boost", C.c_double),
        ("transfer_only", C.c_int), ("num_transfer_times", C.c_int), ("transfer_times", _c_double_p),
        ("hubble_h", C.c_double), ("want_cls", C.c_int), ("transfer_high_precision", C.c_int),
        ("late_phot_switch_boost_min", C.c_double),
        ("src_keep_tau", C.c_double),
        ("transfer_source_modes", C.c_int),
    ]


# every symbol declared in include/cambgpu.h, with its ctypes signature
SIGNATURES = {
    "cambgpu_default_params": (None, [C.POINTER(CambGpuParams)]),
    "cambgpu_tables_create": (C.c_int, [C.POINTER(CambGpuParams), C.POINTER(C.c_void_p)]),
    "cambgpu_tables_view": (C.c_int, [C.c_void_p, C.POINTER(CambGpuTables)]),
    "cambgpu_tables_transfer_view": (C.c_int, [C.c_void_p, C.POINTER(CambGpuTables)]),
    "cambgpu_tables_destroy": (None, [C.c_void_p]),
    "cambgpu_tables_derived": (C.c_int, [C.c_void_p, _c_double_p]),
    "cambgpu_recfast_xe": (C.c_int, [C.c_void_p, _c_double_p, C.c_int, _c_double_p]),
    "cambgpu_conformal_time": (C.c_int, [C.c_void_p, _c_double_p, C.c_int, _c_double_p]),
    "cambgpu_evolve_scalar_sources": (C.c_int, [C.POINTER(CambGpuTables), _c_double_p]),
    "cambgpu_los_flat": (C.c_int, [C.POINTER(CambGpuTables), _c_double_p, _c_double_p]),
    "cambgpu_calc_scal_cls": (C.c_int, [C.POINTER(CambGpuTables), _c_double_p, _c_double_p]),
    "cambgpu_los_flat_noalloc": (C.c_int, [C.POINTER(CambGpuTables), C.c_void_p, C.c_void_p, C.c_void_p]),
    "cambgpu_get_results": (C.c_int, [C.POINTER(CambGpuParams), C.c_int, _c_double_p]),
    "cambgpu_get_results_batch": (C.c_int, [C.POINTER(CambGpuParams), C.c_int, C.c_int, _c_double_p, _c_int_p]),
    "cambgpu_get_spectra_batch": (C.c_int, [C.POINTER(CambGpuParams), C.c_int, C.c_int, _c_double_p, _c_double_p,
                                              _c_double_p, _c_int_p, _c_int_p]),
    "cambgpu_get_transfer_batch": (C.c_int, [C.POINTER(CambGpuParams), C.c_int, C.c_int, C.POINTER(C.c_float),
                                               _c_int_p, _c_double_p, _c_double_p, _c_int_p]),
    "cambgpu_get_results_with_transfers": (C.c_int, [C.POINTER(CambGpuParams), C.c_int, C.c_int, _c_double_p,
                                                       _c_double_p, _c_double_p, _c_int_p, C.c_int,
                                                       C.POINTER(C.c_float), _c_int_p, _c_double_p, _c_double_p,
                                                       _c_int_p]),
    "cambgpu_lensing_range": (C.c_int, [C.POINTER(CambGpuTables), _c_int_p]),
    "cambgpu_batch_prepare": (C.c_int, [C.POINTER(CambGpuParams), C.c_int]),
    "cambgpu_batch_prepare_shared": (C.c_int, [C.POINTER(CambGpuParams), C.c_int, _c_int_p]),
    "cambgpu_tables_share_grids": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, _c_int_p]),
    "cambgpu_batch_run": (C.c_int, [_c_double_p]),
    "cambgpu_batch_fetch": (C.c_int, [C.c_int, _c_double_p]),
    "cambgpu_batch_release": (None, []),
    "cambgpu_batch_spectra_from_transfer": (C.c_int, [_c_double_p, _c_double_p, _c_double_p, _c_double_p, C.c_int,
                                                        _c_double_p, _c_double_p, _c_double_p, _c_int_p]),
    "cambgpu_set_ode_team": (C.c_int, [C.c_int]),
    "cambgpu_set_ode_launch": (C.c_int, [C.c_int, C.c_int]),
    "cambgpu_set_ode_schedule": (C.c_int, [C.c_int]),
    "cambgpu_prepare_tables": (C.c_int, [C.POINTER(CambGpuParams), C.c_int, C.POINTER(C.c_void_p), _c_int_p]),
    "cambgpu_get_spectra_prepared": (C.c_int, [C.c_void_p, C.c_int, _c_double_p, _c_double_p, _c_double_p, _c_int_p,
                                               _c_int_p]),
    "cambgpu_free_prepared": (None, [C.c_void_p]),
    "cambgpu_set_precision": (C.c_int, [C.c_int]),
    "cambgpu_get_precision": (C.c_int, []),
    "cambgpu_autotune_ode": (C.c_int, [C.POINTER(CambGpuParams), C.c_int, _c_int_p, _c_double_p]),
    "cambgpu_last_timings": (C.c_int, [_c_double_p]),
    "cambgpu_last_host_timings": (C.c_int, [_c_double_p]),
    "cambgpu_last_ode_evals": (C.c_longlong, []),
    "cambgpu_last_transfer_bytes": (C.c_int, [C.POINTER(C.c_longlong)]),
    "cambgpu_probe_fp64_tflops": (C.c_int, [_c_double_p]),
    "cambgpu_probe_fp64_pipe": (C.c_int, [C.c_int, C.c_int, C.c_int, _c_double_p]),
    "cambgpu_gemm_bf16x3": (C.c_int, [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int, C.c_int,
                                      C.POINTER(C.c_float)]),
    "cambgpu_kernel_launches": (C.c_longlong, [C.c_int]),
    "cambgpu_last_error": (C.c_char_p, []),
}

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Loads the in-tree libcambgpu.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"libcambgpu.so not built ({path})")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class CAMBError(Exception):
    """Error raised when the library returns a non-zero code (camb/_config.py CAMBError)."""


def check(rc):
    if rc != 0:
        msg = load().cambgpu_last_error().decode(errors="replace")
        raise CAMBError(f"error {rc}: {msg}")


def dptr(a):
    return a.ctypes.data_as(_c_double_p)


def iptr(a):
    return a.ctypes.data_as(_c_int_p)


def default_params():
    p = CambGpuParams()
    load().cambgpu_default_params(C.byref(p))
    return p


class Tables:
    """Host tables of one cosmology (a handle of cambgpu_tables_create)."""

    def __init__(self, params):
        self._lib = load()
        self.params = params
        h = C.c_void_p()
        check(self._lib.cambgpu_tables_create(C.byref(params), C.byref(h)))
        self.handle = h
        self.view = CambGpuTables()
        check(self._lib.cambgpu_tables_view(h, C.byref(self.view)))

    def transfer_view(self):
        """The transfer-function half of a run that wants the CMB and transfer functions."""
        v = CambGpuTables()
        check(self._lib.cambgpu_tables_transfer_view(self.handle, C.byref(v)))
        return v

    def close(self):
        if self.handle:
            self._lib.cambgpu_tables_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def derived(self):
        out = np.zeros(8)
        check(self._lib.cambgpu_tables_derived(self.handle, dptr(out)))
        keys = ["tau0", "DMt0", "taurst", "taurend", "tau_maxvis", "zre", "z_drag", "scale"]
        return dict(zip(keys, out))

    def recfast_xe(self, z):
        z = np.ascontiguousarray(z, dtype=np.float64)
        out = np.zeros_like(z)
        check(self._lib.cambgpu_recfast_xe(self.handle, dptr(z), len(z), dptr(out)))
        return out

    def conformal_time(self, z):
        """Conformal time from the big bang to redshift z in Mpc (CAMBdata.conformal_time)."""
        z = np.ascontiguousarray(np.atleast_1d(z), dtype=np.float64)
        out = np.zeros_like(z)
        check(self._lib.cambgpu_conformal_time(self.handle, dptr(z), len(z), dptr(out)))
        return out

    def array(self, name, n):
        p = getattr(self.view, name)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    @property
    def ls(self):
        return np.ctypeslib.as_array(self.view.ls, shape=(self.view.nl,)).copy()

    @property
    def q_evolve(self):
        return self.array("q_evolve", self.view.nk)

    @property
    def q_int(self):
        return self.array("q_int", self.view.nq)

    @property
    def tau_points(self):
        return self.array("tau_points", self.view.ntau)

    def modes(self):
        v = self.view
        return [(v.modes[i].q, v.modes[i].taustart, v.modes[i].tight_switch_tau, v.modes[i].lmaxg,
                 v.modes[i].lmaxgpol, v.modes[i].lmaxnr) for i in range(v.nk)]

    def shapes(self):
        v = self.view
        return dict(src=(v.ntau, v.nsrc, v.nk), delta=(v.nq, v.nl, v.nsrc), icl=(v.nl, 6))

    # ---- GPU hot path through the C ABI ----
    def evolve_sources_gpu(self):
        s = self.shapes()["src"]
        out = np.zeros(s)
        check(self._lib.cambgpu_evolve_scalar_sources(C.byref(self.view), dptr(out)))
        return out

    def los_gpu(self, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        out = np.zeros(self.shapes()["delta"])
        check(self._lib.cambgpu_los_flat(C.byref(self.view), dptr(src), dptr(out)))
        return out

    def cls_gpu(self, delta):
        delta = np.ascontiguousarray(delta, dtype=np.float64)
        out = np.zeros(self.shapes()["icl"])
        check(self._lib.cambgpu_calc_scal_cls(C.byref(self.view), dptr(delta), dptr(out)))
        return out
