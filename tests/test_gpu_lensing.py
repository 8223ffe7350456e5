"""GPU parity of the C_l interpolation to every l (templated spline), the lensing of the
C_l (CorrFuncFullSkyApodized) and the lensing-potential output, through
cambgpu_get_spectra_batch, against the oracle on the same inputs.  Tolerance: 1e-5
relative on TT, EE, BB and on TE / sqrt(TT EE), as for the C_l."""
import numpy as np
import pytest

from camb_gb300 import _lib
from oracle import oracle as orc
from tests.cosmologies import draws, fiducial

pytestmark = pytest.mark.gpu


def oracle_spectra(p):
    T = _lib.Tables(p)
    icl = orc.cls(T, orc.los(T, orc.evolve_sources(T)))
    allc = orc.interpolate_cls(T.ls, icl, T.view.cl_template_scale)
    lensed = orc.lens_cls(allc[:, :4], T.ls, p.max_l) if p.do_lensing else None
    return T, allc, lensed


def gpu_spectra(ps, lmax_out):
    lib = _lib.load()
    n = len(ps)
    arr = (_lib.CambGpuParams * n)(*ps)
    unl = np.zeros((n, lmax_out + 1, 4))
    lens = np.zeros((n, lmax_out + 1, 4))
    pot = np.zeros((n, lmax_out + 1, 3))
    lml = np.zeros(n, dtype=np.int32)
    st = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_spectra_batch(arr, n, lmax_out, _lib.dptr(unl), _lib.dptr(lens), _lib.dptr(pot),
                                             _lib.iptr(lml), _lib.iptr(st)))
    assert not st.any()
    return unl, lens, pot, lml


def check4(got, ref, lo, hi, tol=1e-5, bb=True):
    s = slice(lo, hi + 1)
    assert np.max(np.abs(got[s, 0] / ref[s, 0] - 1)) < tol
    assert np.max(np.abs(got[s, 1] / ref[s, 1] - 1)) < tol
    if bb:
        assert np.max(np.abs(got[s, 2] / ref[s, 2] - 1)) < tol
    assert np.max(np.abs(got[s, 3] - ref[s, 3]) / np.sqrt(ref[s, 0] * ref[s, 1])) < tol


def as_tebt(allc):
    out = np.zeros((allc.shape[0], 4))
    out[:, 0], out[:, 1], out[:, 3] = allc[:, 0], allc[:, 1], allc[:, 2]
    return out


def test_unlensed_every_l_matches_oracle():
    p = fiducial(1000)
    T, allc, _ = oracle_spectra(p)
    unl, _, _, lml = gpu_spectra([p], 1000)
    check4(unl[0], as_tebt(allc), 2, 1000, bb=False)
    assert lml[0] == 0


def test_lensed_and_potential_match_oracle():
    p = fiducial(1000, lensing=True)
    T, allc, lensed = oracle_spectra(p)
    unl, lens, pot, lml = gpu_spectra([p], p.max_l)
    n = lensed.shape[0] - 1
    assert lml[0] == n == orc.lensing_lrange(T.ls, p.max_l)[1]
    check4(unl[0], as_tebt(allc), 2, p.max_l, bb=False)
    check4(lens[0], lensed, 2, n)
    assert not lens[0][n + 1:].any()
    ell = np.arange(2, p.max_l + 1, dtype=np.float64)
    pp = allc[2:, 3] * ((ell + 1) / ell) ** 2 / (2 * np.pi)
    assert np.max(np.abs(pot[0][2:, 0] / pp - 1)) < 1e-5
    assert np.all(np.isfinite(pot[0]))


def test_lensed_batch_with_massive_neutrinos_and_unlensed_members():
    ps = draws(3, seed=21, lmax=600, mnu_max=0.2)
    for p in ps[:2]:
        p.do_lensing = 1
        p.max_l = 800
        p.max_eta_k = 800 * 2.5
    unl, lens, pot, lml = gpu_spectra(ps, 800)
    for i, p in enumerate(ps):
        T, allc, lensed = oracle_spectra(p)
        check4(unl[i], as_tebt(allc), 2, p.max_l, bb=False)
        if p.do_lensing:
            assert lml[i] == lensed.shape[0] - 1
            check4(lens[i], lensed, 2, lml[i])
        else:
            assert lml[i] == 0 and not lens[i].any() and not pot[i].any()


def test_python_surface_lensed_spectra():
    from camb_gb300 import model, results
    cp = model.set_params(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.06, tau=0.06, As=2.1e-9, ns=0.965, lmax=600)
    assert cp.DoLensing and cp.max_l == 800
    r = results.get_results(cp)
    d = r.get_cmb_power_spectra(CMB_unit="muK")
    assert set(d) == {"total", "unlensed_scalar", "unlensed_total", "lensed_scalar", "tensor", "lens_potential"}
    n = d["lensed_scalar"].shape[0] - 1
    assert n == r._lmax_lensed >= 600
    assert np.allclose(d["total"], d["lensed_scalar"])
    tt = d["lensed_scalar"][2:n + 1, 0]
    assert np.all(tt > 0) and 5000 < tt[218] < 6500  # first acoustic peak near l=220, muK^2
    assert d["lens_potential"][10, 0] > 0
