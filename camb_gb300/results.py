"""Results object, mirroring the reference's camb/results.py CAMBdata C_l getters
(results.py:417-508, 1227-1290): unlensed and lensed scalar spectra and the lensing
potential, all computed on the GPU through cambgpu_get_spectra_batch."""
import copy
import ctypes as C

import numpy as np

from . import _lib


def save_cmb_power_array(filename, array, labels, lmin=0):
    """Writes a zero-based (lmax+1, ncol) C_l array as text, one line per L from lmin: the
    L column ("%4u"), then each column in "%12.7e", under a "# L <labels>" header line
    (results.py:62-82, the format the reference's CAMB text outputs use)."""
    array = np.asarray(array)
    cols = labels.split() if isinstance(labels, str) else list(labels)
    ell = np.arange(lmin, array.shape[0], dtype=np.float64)[:, None]
    header = " L " + " ".join(f"{c:13s}" for c in cols)
    np.savetxt(filename, np.hstack((ell, array[lmin:])), fmt=["%4u"] + ["%12.7e"] * array.shape[1], header=header)


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

    def save_cmb_power_spectra(self, filename, lmax=None, CMB_unit="muK"):
        """results.py:459-472: total (lensed when lensing) l(l+1)C_l/2pi, then the lensing
        potential and its crosses: columns L TT EE BB TE PP PT PE."""
        lmax = self._lmax_setting(lmax, False)
        cmb = self.get_total_cls(lmax, CMB_unit=CMB_unit)
        pot = self.get_lens_potential_cls(lmax, CMB_unit=CMB_unit)
        save_cmb_power_array(filename, np.hstack((cmb, pot)), "TT EE BB TE PP PT PE")

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


def _run_prepared(handle, params_list, lmax_out):
    lib = _lib.load()
    n = len(params_list)
    cls = np.zeros((n, lmax_out + 1, 4))
    lens = any(p.DoLensing for p in params_list)
    lensed = np.zeros((n, lmax_out + 1, 4)) if lens else None
    pot = np.zeros((n, lmax_out + 1, 3)) if lens else None
    lml = np.zeros(n, dtype=np.int32)
    status = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_spectra_prepared(handle, lmax_out, _lib.dptr(cls),
                                                _lib.dptr(lensed) if lens else None,
                                                _lib.dptr(pot) if lens else None, _lib.iptr(lml), _lib.iptr(status)))
    return [CAMBdata(p, cls[i], lensed[i] if lens and p.DoLensing else None,
                     pot[i] if lens and p.DoLensing else None, int(lml[i])) for i, p in enumerate(params_list)]


def _prepare(params_list):
    lib = _lib.load()
    n = len(params_list)
    arr = (_lib.CambGpuParams * n)(*[p.to_struct() for p in params_list])
    handle = C.c_void_p()
    status = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_prepare_tables(arr, n, C.byref(handle), _lib.iptr(status)))
    return handle


def get_results_stream(batches, lmax_out=None):
    """get_results_batch over a sequence of batches, pipelined: while the device runs one
    batch, a host thread builds the next batch's tables (cambgpu_prepare_tables) and
    releases the previous batch's.  Yields each batch's list of CAMBdata in order."""
    from concurrent.futures import ThreadPoolExecutor
    lib = _lib.load()
    it = iter(batches)
    cur = next(it, None)
    if cur is None:
        return
    with ThreadPoolExecutor(1) as ex:
        fut = ex.submit(_prepare, cur)
        try:
            while cur is not None:
                handle = fut.result()
                fut = None
                nxt = next(it, None)
                if nxt is not None:
                    fut = ex.submit(_prepare, nxt)
                try:
                    lmax = max(p.max_l for p in cur) if lmax_out is None else lmax_out
                    if any(p.WantTransfer for p in cur):  # transfer functions: the batch path
                        out = get_results_batch(cur, lmax)
                    else:
                        out = _run_prepared(handle, cur, lmax)
                finally:
                    ex.submit(lib.cambgpu_free_prepared, handle)  # released on the host thread
                yield out
                cur = nxt
        finally:
            if fut is not None:  # the consumer stopped early: release the prepared batch
                try:
                    lib.cambgpu_free_prepared(fut.result())
                except _lib.CAMBError:
                    pass


def _run_both(params_list, lmax_out):
    """WantCls and WantTransfer together, as the reference's single evolution
    (cambgpu_get_results_with_transfers: one transfer-path launch stores each source
    mode's CMB sources at the source times and its transfer variables at the transfer
    times; the projection and C_l follow on those sources), one CAMBdataMatter per
    cosmology."""
    lib = _lib.load()
    n = len(params_list)
    nz = params_list[0].Transfer.PK_num_redshifts
    if any(p.Transfer.PK_num_redshifts != nz for p in params_list):
        raise _lib.CAMBError("a transfer batch needs the same number of redshifts")
    arr = (_lib.CambGpuParams * n)(*[p.to_struct() for p in params_list])
    cls = np.zeros((n, lmax_out + 1, 4))
    lens = any(p.DoLensing for p in params_list)
    lensed = np.zeros((n, lmax_out + 1, 4)) if lens else None
    pot = np.zeros((n, lmax_out + 1, 3)) if lens else None
    lml = np.zeros(n, dtype=np.int32)
    nq_max = 4096
    tr = np.zeros((n, nz, nq_max, 13), dtype=np.float32)
    nq = np.zeros(n, dtype=np.int32)
    s8 = np.zeros((n, nz))
    sv = np.zeros((n, nz))
    st = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_results_with_transfers(
        arr, n, lmax_out, _lib.dptr(cls), _lib.dptr(lensed) if lens else None, _lib.dptr(pot) if lens else None,
        _lib.iptr(lml), nq_max, tr.ctypes.data_as(C.POINTER(C.c_float)), _lib.iptr(nq), _lib.dptr(s8),
        _lib.dptr(sv), _lib.iptr(st)))
    out = []
    for i, p in enumerate(params_list):
        td = np.ascontiguousarray(tr[i, :, : nq[i], :].transpose(2, 1, 0))  # [13, nq, nz]
        q = td[0, :, 0].astype(np.float64) * p.H0 / 100
        r = CAMBdataMatter(p, MatterTransferData(td, q, s8[i], sv[i]))
        r._cls = cls[i]
        r._lensed = lensed[i] if lens and p.DoLensing else None
        r._pot = pot[i] if lens and p.DoLensing else None
        r._lmax_lensed = int(lml[i])
        out.append(r)
    return out


def get_results(params, lmax_out=None):
    """camb.get_results (camb.py:47-61): one cosmology through the GPU pipeline -- the CMB
    spectra, the matter transfer functions (WantTransfer), or both."""
    return get_results_batch([params], lmax_out)[0]


def get_results_batch(params_list, lmax_out=None):
    """Many cosmologies in one persistent launch per stage."""
    want_cls = [p.WantCls for p in params_list]
    want_tr = [p.WantTransfer for p in params_list]
    lmax = max(p.max_l for p in params_list) if lmax_out is None else lmax_out
    if all(want_tr) and not any(want_cls):
        return _run_transfer(params_list)
    if all(want_tr) and all(want_cls):
        return _run_both(params_list, lmax)
    if any(want_tr):
        raise _lib.CAMBError("a batch either wants transfer functions in every member or in none")
    return _run(params_list, lmax)


_PROJECTIONS = {"fp64": 0, "mixed": 1, "tensor": 2}


def get_results_batch_shared(params_list, lmax_out=None, projection="tensor"):
    """A batch of CMB cosmologies on grids shared by the whole batch
    (cambgpu_batch_prepare_shared: one comoving-distance grid, one source k grid, one
    integration q grid and one Bessel table for every member; no counterpart in the
    reference, where each cosmology has its own grids).  `projection` chooses the
    arithmetic of the line-of-sight projection: "tensor" (split hi/lo BF16 products on the
    tensor cores, FP32 accumulation), "mixed" (FP32) or "fp64".  All members share one l
    sampling and one set of sources; the C_l differ from get_results_batch by the shared
    grids' resampling (a few 1e-4 at high l), and the tensor and mixed forms from the FP64
    one on the same grids by ~1e-5.  Returns one CAMBdata per cosmology."""
    if projection not in _PROJECTIONS:
        raise _lib.CAMBError(f"projection must be one of {sorted(_PROJECTIONS)}")
    if any(p.WantTransfer or not p.WantCls for p in params_list):
        raise _lib.CAMBError("shared grids are for CMB spectra only (WantCls, no WantTransfer)")
    lib = _lib.load()
    params = list(params_list)
    n = len(params)
    lmax = max(p.max_l for p in params) if lmax_out is None else lmax_out
    arr = (_lib.CambGpuParams * n)(*[p.to_struct() for p in params])
    prev = lib.cambgpu_get_precision()
    _ResidentBatch.generation += 1  # the arena now holds this batch
    _lib.check(lib.cambgpu_batch_prepare_shared(arr, n, None))
    try:
        _lib.check(lib.cambgpu_set_precision(_PROJECTIONS[projection]))
        _lib.check(lib.cambgpu_batch_run(None))
        cls = np.zeros((n, lmax + 1, 4))
        lensed = np.zeros((n, lmax + 1, 4))
        pot = np.zeros((n, lmax + 1, 3))
        lml = np.zeros(n, dtype=np.int32)
        _lib.check(lib.cambgpu_batch_spectra_from_transfer(None, None, None, None, lmax, _lib.dptr(cls),
                                                           _lib.dptr(lensed), _lib.dptr(pot), _lib.iptr(lml)))
    finally:
        lib.cambgpu_set_precision(prev)
        lib.cambgpu_batch_release()
    return [CAMBdata(p, cls[i], lensed[i] if p.DoLensing else None, pot[i] if p.DoLensing else None,
                     int(lml[i])) for i, p in enumerate(params)]


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


def get_matter_power_interpolator(params, zmin=0.0, zmax=10.0, nz_step=100, zs=None, kmax=10.0, nonlinear=True,
                                  var1=None, var2=None, hubble_units=True, k_hunit=True, return_z_k=False,
                                  k_per_logint=None, log_interp=True, extrap_kmax=None):
    """camb.get_matter_power_interpolator: transfer functions of a copy of params at zs
    (default nz_step redshifts from zmin to zmax, evenly spaced in ln(1 + z - zmin)) to
    kmax (1/Mpc), then CAMBdataMatter.get_matter_power_interpolator.  Linear power (the
    reference also switches the non-linear model off here); the CMB is not computed."""
    pars = copy.deepcopy(params)
    if zs is None:
        zs = zmin + np.exp(np.log(zmax - zmin + 1) * np.linspace(0, 1, nz_step)) - 1
    pars.set_matter_power(redshifts=list(zs), kmax=kmax, k_per_logint=k_per_logint)
    pars.WantCls = False
    return get_results(pars).get_matter_power_interpolator(nonlinear, var1, var2, hubble_units, k_hunit, return_z_k,
                                                           log_interp, extrap_kmax)


def get_transfer_functions(params):
    """camb.get_transfer_functions (camb.py:64-79) for the scalar CMB path."""
    return CAMBdataTransfers(_ResidentBatch([params]), 0)


def get_transfer_functions_batch(params_list):
    batch = _ResidentBatch(params_list)
    return [CAMBdataTransfers(batch, i) for i in range(len(params_list))]


class MatterTransferData:
    """MatterTransferData (results.f90, camb/results.py get_matter_transfer_data):
    transfer_data[13, nq, nz] single precision, q (1/Mpc), sigma_8, sigma2_vdelta_8."""

    def __init__(self, transfer_data, q, sigma_8, sigma2_vdelta_8):
        self.transfer_data = transfer_data
        self.q = q
        self.sigma_8 = sigma_8
        self.sigma2_vdelta_8 = sigma2_vdelta_8
        self.nq = len(q)


class CAMBdataMatter(CAMBdata):
    """Results of a transfer-function run (WantTransfer, WantCls off): sigma8, f sigma8,
    the transfer functions and the linear matter power spectrum (camb/results.py:806-998)."""

    def __init__(self, params, mtd):
        super().__init__(params, np.zeros((params.max_l + 1, 4)))
        self._mtd = mtd

    def get_matter_transfer_data(self):
        return self._mtd

    def get_sigma8(self):
        return np.array(self._mtd.sigma_8)

    def get_sigma8_0(self):
        if self.Params.Transfer.PK_redshifts[-1] > 1e-5:
            raise _lib.CAMBError("sigma8 requested at z=0, but P(z=0) not calculated")
        return self.get_sigma8()[-1]

    def get_fsigma8(self):
        return self._mtd.sigma2_vdelta_8 / self._mtd.sigma_8

    def get_matter_power_spectrum(self, minkh=1e-4, maxkh=1.0, npoints=100, var1=None, var2=None, **kwargs):
        """camb/results.py get_matter_power_spectrum (results.py:1000-1048), linear:
        kh (npoints values log-spaced from minkh to maxkh), z increasing, PK[z, kh] in
        (Mpc/h)^3, splined from the transfer functions (matter_power_on_log_grid)."""
        return _matter_power_spectrum(self.Params, self._mtd.transfer_data, minkh, maxkh, npoints, var1, var2)

    def get_matter_power_interpolator(self, nonlinear=True, var1=None, var2=None, hubble_units=True, k_hunit=True,
                                      return_z_k=False, log_interp=True, extrap_kmax=None, silent=False):
        """camb/results.py get_matter_power_interpolator: a spline of P(z, k/h) (or of k) through
        the transfer-grid power at the transfer redshifts -- cubic in ln k, of degree
        min(nz - 1, 3) in z, of ln(sign P) unless P changes sign; with extrap_kmax, ln P is
        continued as a power law of the last interval's slope to extrap_kmax.  Evaluate with
        .P(z, kh) (or call it with (z, ln kh) for the interpolated value itself).  The power
        is linear: halo-model corrections are not part of this package, and nonlinear=True
        returns the linear spectrum as the reference does for a model without them."""
        kh, zs, pk = self.get_linear_matter_power_spectrum(var1, var2, hubble_units)
        if not k_hunit:
            kh = kh * self.Params.H0 / 100
        return MatterPowerInterpolator(zs, kh, pk, log_interp, extrap_kmax, return_z_k)

    def get_linear_matter_power_spectrum(self, var1=None, var2=None, hubble_units=True, k_hunit=True, **kwargs):
        """Transfer_GetUnsplinedPower (results.f90:3472-3513) on the transfer k grid:
        returns k/h (or k), z increasing, PK[z, k]."""
        td = self._mtd.transfer_data
        s1 = 6 if var1 is None else int(var1) - 1
        s2 = 6 if var2 is None else int(var2) - 1
        ip = self.Params.InitPower
        h = self.Params.H0 / 100
        kh = td[0, :, 0].astype(np.float64)
        k = kh * h
        lnrat = np.log(k / ip.pivot_scalar)
        power = ip.As * np.exp(lnrat * (ip.ns - 1 + lnrat * (ip.nrun / 2)))
        nz = td.shape[2]
        pk = np.empty((nz, len(k)))
        for zix in range(nz):
            it = nz - 1 - zix
            pk[zix] = td[s1, :, it].astype(np.float64) * td[s2, :, it] * k * np.pi * 2 * np.pi * power
        if hubble_units:
            pk *= h ** 3
        z = np.array(self.Params.Transfer.PK_redshifts[::-1], dtype=np.float64)
        return (kh if k_hunit else k), z, pk


class _PK:
    """P(z, k) spline built by MatterPowerInterpolator."""

    def __init__(self, zs, logk, vals, islog, sign):
        from scipy.interpolate import CubicSpline, RectBivariateSpline
        self.islog, self.logsign = islog, sign
        self.zmin, self.zmax = float(np.min(zs)), float(np.max(zs))
        self._zs = np.asarray(zs, dtype=np.float64)
        if len(zs) > 1:
            self._s2 = RectBivariateSpline(self._zs, logk, vals, kx=min(len(zs) - 1, 3), ky=min(len(logk) - 1, 3))
            self._s1 = None
        else:
            self._s2 = None
            self._s1 = CubicSpline(logk, vals[0])

    def __call__(self, z, logk, grid=None):
        """The interpolated value (ln(sign P) when islog) at (z, ln k)."""
        if grid is None:
            grid = not np.isscalar(z) and not np.isscalar(logk)
        if self._s2 is not None:
            return self._s2(z, logk, grid=grid)
        if not np.allclose(z, self._zs[0]):
            raise _lib.CAMBError(f"P(z,k) requested at z={z}, but only computed for z={self._zs[0]:g}")
        return self._s1(logk)

    def P(self, z, kh, grid=None):
        v = self(z, np.log(kh), grid=grid)
        return self.logsign * np.exp(v) if self.islog else v


def MatterPowerInterpolator(zs, kh, pk, log_interp=True, extrap_kmax=None, return_z_k=False):
    """The spline of get_matter_power_interpolator from P[z, kh] on the transfer grid."""
    zs = np.asarray(zs, dtype=np.float64)
    kh = np.asarray(kh, dtype=np.float64)
    sign = 1.0
    if log_interp and np.any(pk <= 0):
        if np.all(pk < 0):
            sign = -1.0
        else:
            log_interp = False
    vals = np.log(sign * pk) if log_interp else np.array(pk, dtype=np.float64)
    logk = np.log(kh)
    kmax = kh[-1]
    if extrap_kmax and extrap_kmax > kmax:
        if not log_interp:
            raise _lib.CAMBError("extrap_kmax needs log interpolation (the power changes sign)")
        # power law with the last interval's slope, on two nodes: one a tenth of the way back
        # from extrap_kmax (slope scaled by 0.9) and one at extrap_kmax
        span = np.log(extrap_kmax) - logk[-1]
        slope = (vals[:, -1] - vals[:, -2]) / (logk[-1] - logk[-2])
        vals = np.hstack((vals, (vals[:, -1] + 0.9 * slope * span)[:, None], (vals[:, -1] + slope * span)[:, None]))
        logk = np.hstack((logk, np.log(extrap_kmax) - 0.1 * span, np.log(extrap_kmax)))
    res = _PK(zs, logk, vals, log_interp, sign)
    res.kmin, res.kmax = float(np.min(kh)), float(kmax)
    return (res, zs, kh) if return_z_k else res


def _natural_spline_d2(x, y):
    """Second derivatives of the natural cubic spline through (x, y) (zero at both ends),
    by the tridiagonal recurrence; y may carry trailing columns."""
    n = len(x)
    d2 = np.zeros_like(y)
    if n < 3:
        return d2
    u = np.zeros_like(y)
    for i in range(1, n - 1):
        sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1])
        p = sig * d2[i - 1] + 2.0
        d2[i] = (sig - 1.0) / p
        slope = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])
        u[i] = (6.0 * slope / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p
    for i in range(n - 2, -1, -1):
        d2[i] = d2[i] * d2[i + 1] + u[i]
    return d2


def matter_power_on_log_grid(kh, t1, t2, h, init_power, minkh, dlnkh, npoints):
    """Transfer_GetMatterPowerD (results.f90:3841-3948), linear: P(k/h) at npoints values
    spaced by dlnkh in ln(k/h) from minkh, in (Mpc/h)^3, from the transfer functions t1, t2
    on the transfer grid kh (k/h) of one redshift.  The transfer part T1 T2 k 2pi^2 h^3 is
    splined in ln(k/h) -- in its logarithm when it has one sign, a natural cubic spline --
    and extrapolated linearly in ln k past the last node (below the first node the result is
    the floor exp(-30)); the primordial power multiplies the interpolated value."""
    kh = np.asarray(kh, dtype=np.float64)
    x = np.log(kh)
    mp = np.asarray(t1, dtype=np.float64) * np.asarray(t2, dtype=np.float64) * kh * h * np.pi * 2 * np.pi * h ** 3
    sign, log_interp = 1.0, True
    if np.any(mp <= 0):
        if np.all(mp < 0):
            sign = -1.0
        else:
            log_interp = False
    if log_interp:
        mp = np.log(sign * mp)
    d2 = _natural_spline_d2(x, mp)
    out = np.empty(npoints)
    xi = np.log(minkh) + dlnkh * np.arange(npoints)
    n = len(x)
    llo, last = 0, npoints
    for il in range(npoints):
        if xi[il] < x[0]:
            out[il] = -30.0
            continue
        while llo < n - 1 and xi[il] > x[llo + 1]:
            llo += 1
        if llo == n - 1:
            last = il
            break
        ho = x[llo + 1] - x[llo]
        a0 = (x[llo + 1] - xi[il]) / ho
        b0 = (xi[il] - x[llo]) / ho
        out[il] = a0 * mp[llo] + b0 * mp[llo + 1] + ((a0 ** 3 - a0) * d2[llo] + (b0 ** 3 - b0) * d2[llo + 1]) * ho ** 2 / 6
    for il in range(last, npoints):  # linear extrapolation in the logarithm
        out[il] = 2 * out[il - 1] - out[il - 2]
    if log_interp:
        out = sign * np.exp(np.maximum(-30.0, out))
    k = np.exp(xi) * h
    lnrat = np.log(k / init_power.pivot_scalar)
    return out * init_power.As * np.exp(lnrat * (init_power.ns - 1 + lnrat * (init_power.nrun / 2)))


def _matter_power_spectrum(params, td, minkh, maxkh, npoints, var1, var2):
    if not npoints >= 2:
        raise _lib.CAMBError("Need at least two points in get_matter_power_spectrum")
    s1 = 6 if var1 is None else int(var1) - 1
    s2 = 6 if var2 is None else int(var2) - 1
    h = params.H0 / 100
    nz = td.shape[2]
    dlnkh = (np.log(maxkh) - np.log(minkh)) / (npoints - 1)
    pk = np.empty((nz, npoints))
    for zix in range(nz):
        it = nz - 1 - zix  # increasing z: the transfer times are stored in decreasing z
        pk[zix] = matter_power_on_log_grid(td[0, :, it], td[s1, :, it], td[s2, :, it], h, params.InitPower, minkh,
                                           dlnkh, npoints)
    z = np.array(params.Transfer.PK_redshifts[::-1], dtype=np.float64)
    return minkh * np.exp(np.arange(npoints) * dlnkh), z, pk


def _run_transfer(params_list):
    lib = _lib.load()
    n = len(params_list)
    nz = params_list[0].Transfer.PK_num_redshifts
    if any(p.Transfer.PK_num_redshifts != nz for p in params_list):
        raise _lib.CAMBError("a transfer batch needs the same number of redshifts")
    arr = (_lib.CambGpuParams * n)(*[p.to_struct() for p in params_list])
    nq_max = 4096
    tr = np.zeros((n, nz, nq_max, 13), dtype=np.float32)
    nq = np.zeros(n, dtype=np.int32)
    s8 = np.zeros((n, nz))
    sv = np.zeros((n, nz))
    st = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_transfer_batch(arr, n, nq_max, tr.ctypes.data_as(C.POINTER(C.c_float)),
                                              _lib.iptr(nq), _lib.dptr(s8), _lib.dptr(sv), _lib.iptr(st)))
    out = []
    for i, p in enumerate(params_list):
        td = np.ascontiguousarray(tr[i, :, : nq[i], :].transpose(2, 1, 0))  # [13, nq, nz]
        q = td[0, :, 0].astype(np.float64) * p.H0 / 100
        out.append(CAMBdataMatter(p, MatterTransferData(td, q, s8[i], sv[i])))
    return out
