"""Results object, mirroring the reference's camb/results.py CAMBdata C_l getters
(results.py:417-508, 1227-1290) for the unlensed scalar spectra."""
import ctypes as C

import numpy as np

from . import _lib


class CAMBdata:
    def __init__(self, params, cls):
        self.Params = params
        self._cls = cls  # (lmax+1, 4) l(l+1)C_l/2pi, dimensionless: TT EE BB TE

    def _scale(self, cls, lmax, CMB_unit, raw_cl):
        lmax = self._cls.shape[0] - 1 if lmax is None else lmax
        out = np.array(cls[: lmax + 1], copy=True)
        if CMB_unit is not None:
            if isinstance(CMB_unit, str):
                if CMB_unit == "muK":
                    CMB_unit = (self.Params.TCMB * 1e6) ** 2
                elif CMB_unit == "K":
                    CMB_unit = self.Params.TCMB ** 2
                else:
                    raise ValueError("unknown CMB_unit")
            out *= CMB_unit
        if raw_cl:
            ell = np.arange(out.shape[0], dtype=np.float64)
            fac = np.zeros_like(ell)
            fac[1:] = 2 * np.pi / (ell[1:] * (ell[1:] + 1))
            out *= fac[:, None]
        return out

    def get_unlensed_scalar_cls(self, lmax=None, CMB_unit=None, raw_cl=False):
        return self._scale(self._cls, lmax, CMB_unit, raw_cl)

    def get_cmb_power_spectra(self, params=None, lmax=None, spectra=("unlensed_scalar",), CMB_unit=None,
                              raw_cl=False):
        out = {}
        for s in spectra:
            if s in ("unlensed_scalar", "unlensed_total", "total"):
                out[s] = self.get_unlensed_scalar_cls(lmax, CMB_unit, raw_cl)
            else:
                raise ValueError(f"spectrum {s} is not produced by the GPU scalar path")
        return out


def get_results(params, lmax_out=None):
    """camb.get_results (camb.py:47-61): one cosmology through the GPU pipeline."""
    lib = _lib.load()
    lmax_out = params.max_l if lmax_out is None else lmax_out
    s = params.to_struct()
    cls = np.zeros((lmax_out + 1, 4))
    _lib.check(lib.cambgpu_get_results(C.byref(s), lmax_out, _lib.dptr(cls)))
    return CAMBdata(params, cls)


def get_results_batch(params_list, lmax_out=None):
    """Many cosmologies in one persistent launch per stage."""
    lib = _lib.load()
    n = len(params_list)
    lmax_out = max(p.max_l for p in params_list) if lmax_out is None else lmax_out
    arr = (_lib.CambGpuParams * n)(*[p.to_struct() for p in params_list])
    cls = np.zeros((n, lmax_out + 1, 4))
    status = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_results_batch(arr, n, lmax_out, _lib.dptr(cls), _lib.iptr(status)))
    return [CAMBdata(p, cls[i]) for i, p in enumerate(params_list)]
