"""Results object, mirroring the reference's camb/results.py CAMBdata C_l getters
(results.py:417-508, 1227-1290): unlensed and lensed scalar spectra and the lensing
potential, all computed on the GPU through cambgpu_get_spectra_batch."""
import ctypes as C

import numpy as np

from . import _lib


class CAMBdata:
    def __init__(self, params, cls, lensed=None, lens_potential=None, lmax_lensed=0):
        self.Params = params
        self._cls = cls  # (lmax+1, 4) l(l+1)C_l/2pi, dimensionless: TT EE BB TE
        self._lensed = lensed
        self._pot = lens_potential  # (lmax+1, 3) PP PT PE
        self._lmax_lensed = lmax_lensed

    def _CMB_unit(self, CMB_unit):
        if isinstance(CMB_unit, str):
            if CMB_unit == "muK":
                return self.Params.TCMB * 1e6
            if CMB_unit == "K":
                return self.Params.TCMB
            raise ValueError("unknown CMB_unit")
        return CMB_unit

    def _lmax_setting(self, lmax, unlensed):
        """results.py:446-457."""
        lmax_calc = self._cls.shape[0] - 1 if (unlensed or not self.Params.DoLensing) else self._lmax_lensed
        return lmax_calc if lmax is None else lmax

    def _scale(self, cls, lmax, CMB_unit, raw_cl, lens_potential=False):
        """results.py:427-444 (_scale_cls)."""
        out = np.zeros((lmax + 1, cls.shape[1]))
        m = min(lmax, cls.shape[0] - 1)
        out[: m + 1] = cls[: m + 1]
        if raw_cl:
            ell = np.arange(1, out.shape[0], dtype=np.float64)
            llp1 = ell * (ell + 1)
            if lens_potential:
                out[1:, 0] /= llp1 ** 2 / (2 * np.pi)
                out[1:, 1:] /= (llp1 ** 1.5 / (2 * np.pi))[:, None]
            else:
                out[1:, :] /= (llp1 / (2 * np.pi))[:, None]
        if CMB_unit is not None:
            u = self._CMB_unit(CMB_unit)
            if lens_potential:
                out[:, 1:] *= u
            else:
                out *= u ** 2
        return out

    def get_unlensed_scalar_cls(self, lmax=None, CMB_unit=None, raw_cl=False):
        return self._scale(self._cls, self._lmax_setting(lmax, True), CMB_unit, raw_cl)

    def get_unlensed_total_cls(self, lmax=None, CMB_unit=None, raw_cl=False):
        return self.get_unlensed_scalar_cls(lmax, CMB_unit, raw_cl)

    def get_lensed_scalar_cls(self, lmax=None, CMB_unit=None, raw_cl=False):
        if self._lensed is None:
            raise _lib.CAMBError("lensed CL have not been calculated (set DoLensing)")
        return self._scale(self._lensed, self._lmax_setting(lmax, False), CMB_unit, raw_cl)

    def get_lens_potential_cls(self, lmax=None, CMB_unit=None, raw_cl=False):
        pot = self._pot if self._pot is not None else np.zeros((self._cls.shape[0], 3))
        return self._scale(pot, self._lmax_setting(lmax, True), CMB_unit, raw_cl, lens_potential=True)

    def get_tensor_cls(self, lmax=None, CMB_unit=None, raw_cl=False):
        return np.zeros((self._lmax_setting(lmax, False) + 1, 4))

    def get_total_cls(self, lmax=None, CMB_unit=None, raw_cl=False):
        if self.Params.DoLensing:
            return self.get_lensed_scalar_cls(lmax, CMB_unit, raw_cl)
        return self.get_unlensed_scalar_cls(lmax, CMB_unit, raw_cl)

    def get_cmb_power_spectra(self, params=None, lmax=None,
                              spectra=("total", "unlensed_scalar", "unlensed_total", "lensed_scalar", "tensor",
                                       "lens_potential"), CMB_unit=None, raw_cl=False):
        """results.py:474-508: every spectrum to the same lmax (the lensed one when lensing)."""
        lmax = self._lmax_setting(lmax, False)
        out = {}
        for s in spectra:
            if s == "lensed_scalar" and not self.Params.DoLensing:
                continue
            out[s] = getattr(self, "get_" + s + "_cls")(lmax, CMB_unit=CMB_unit, raw_cl=raw_cl)
        return out


def _run(params_list, lmax_out):
    lib = _lib.load()
    n = len(params_list)
    arr = (_lib.CambGpuParams * n)(*[p.to_struct() for p in params_list])
    cls = np.zeros((n, lmax_out + 1, 4))
    lens = any(p.DoLensing for p in params_list)
    lensed = np.zeros((n, lmax_out + 1, 4)) if lens else None
    pot = np.zeros((n, lmax_out + 1, 3)) if lens else None
    lml = np.zeros(n, dtype=np.int32)
    status = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_spectra_batch(arr, n, lmax_out, _lib.dptr(cls),
                                             _lib.dptr(lensed) if lens else None,
                                             _lib.dptr(pot) if lens else None, _lib.iptr(lml), _lib.iptr(status)))
    return [CAMBdata(p, cls[i], lensed[i] if lens and p.DoLensing else None,
                     pot[i] if lens and p.DoLensing else None, int(lml[i])) for i, p in enumerate(params_list)]


def get_results(params, lmax_out=None):
    """camb.get_results (camb.py:47-61): one cosmology through the GPU pipeline."""
    return _run([params], params.max_l if lmax_out is None else lmax_out)[0]


def get_results_batch(params_list, lmax_out=None):
    """Many cosmologies in one persistent launch per stage."""
    return _run(params_list, max(p.max_l for p in params_list) if lmax_out is None else lmax_out)


class _ResidentBatch:
    """A batch whose tables and transfer functions stay on the device (one at a time:
    staging another batch retires this one)."""

    generation = 0

    def __init__(self, params_list):
        lib = _lib.load()
        self.params = list(params_list)
        n = len(self.params)
        arr = (_lib.CambGpuParams * n)(*[p.to_struct() for p in self.params])
        _lib.check(lib.cambgpu_batch_prepare(arr, n))
        _lib.check(lib.cambgpu_batch_run(None))
        _ResidentBatch.generation += 1
        self.gen = _ResidentBatch.generation
        self.lmax = max(p.max_l for p in self.params)

    def spectra(self):
        """Recomputes C_l from the resident transfer functions with every member's current
        primordial power."""
        if self.gen != _ResidentBatch.generation:
            raise _lib.CAMBError("these transfer functions are no longer resident on the device")
        lib = _lib.load()
        n = len(self.params)
        As = np.array([p.InitPower.As for p in self.params])
        ns = np.array([p.InitPower.ns for p in self.params])
        nrun = np.array([p.InitPower.nrun for p in self.params])
        piv = np.array([p.InitPower.pivot_scalar for p in self.params])
        cls = np.zeros((n, self.lmax + 1, 4))
        lensed = np.zeros((n, self.lmax + 1, 4))
        pot = np.zeros((n, self.lmax + 1, 3))
        lml = np.zeros(n, dtype=np.int32)
        _lib.check(lib.cambgpu_batch_spectra_from_transfer(_lib.dptr(As), _lib.dptr(ns), _lib.dptr(nrun),
                                                           _lib.dptr(piv), self.lmax, _lib.dptr(cls),
                                                           _lib.dptr(lensed), _lib.dptr(pot), _lib.iptr(lml)))
        return cls, lensed, pot, lml


class CAMBdataTransfers(CAMBdata):
    """CAMBdata from get_transfer_functions: the transfer functions stay on the device and
    power_spectra_from_transfer recomputes the spectra for new primordial power without
    re-evolving (camb/results.py power_spectra_from_transfer, camb.f90:25-58)."""

    def __init__(self, batch, index):
        self._batch, self._index = batch, index
        super().__init__(batch.params[index], None)
        self._refresh(batch.spectra())

    def _refresh(self, out):
        cls, lensed, pot, lml = out
        i = self._index
        self._cls = cls[i][: self.Params.max_l + 1]
        self._lensed = lensed[i] if self.Params.DoLensing else None
        self._pot = pot[i][: self.Params.max_l + 1] if self.Params.DoLensing else None
        self._lmax_lensed = int(lml[i])

    def power_spectra_from_transfer(self, initial_power_params=None, silent=False):
        if initial_power_params is not None:
            self.Params.InitPower = initial_power_params
        self._refresh(self._batch.spectra())


def get_transfer_functions(params):
    """camb.get_transfer_functions (camb.py:64-79) for the scalar CMB path."""
    return CAMBdataTransfers(_ResidentBatch([params]), 0)


def get_transfer_functions_batch(params_list):
    batch = _ResidentBatch(params_list)
    return [CAMBdataTransfers(batch, i) for i in range(len(params_list))]
