"""Parity at the benchmark configurations' full sizes, GPU (FP64 form, through the C ABI)
against the oracle on the same inputs: draws of the batched configuration at lmax 2500
(one massive eigenstate, mnu in [0, 0.2] eV), the lensed 0.06 eV cosmology at lmax 2500
(+200 margin), and its matter transfer functions to kmax = 10 h/Mpc.  Tolerances as for
the smaller cases: sources within 1e-6 of their peak per k-mode, C_l and lensed C_l
within 1e-5 relative (TE against sqrt(TT EE)), transfer variables within 1e-5 of their
peak over k, sigma8 within 1e-9 relative."""
import ctypes as C

import numpy as np
import pytest

from camb_gb300 import _lib
from oracle import oracle as orc
from tests.cosmologies import draws, fiducial
from tests.test_gpu_lensing import as_tebt, check4, gpu_spectra, oracle_spectra

pytestmark = pytest.mark.gpu


def rel_peak(a, b, axis):
    num = np.max(np.abs(a - b), axis=axis)
    den = np.max(np.abs(b), axis=axis)
    m = den > 0
    return float(np.max(num[m] / den[m])) if np.any(m) else 0.0


@pytest.fixture(autouse=True)
def fp64_form():
    lib = _lib.load()
    old = lib.cambgpu_get_precision()
    _lib.check(lib.cambgpu_set_precision(0))
    yield
    lib.cambgpu_set_precision(old)


def test_batched_draws_lmax2500():
    ps = draws(2, seed=1000, lmax=2500, mnu_max=0.2)
    unl, _, _, _ = gpu_spectra(ps, 2500)
    for i, p in enumerate(ps):
        T = _lib.Tables(p)
        src = orc.evolve_sources(T)
        if i == 0:
            assert rel_peak(T.evolve_sources_gpu(), src, axis=0) < 1e-6
        icl = orc.cls(T, orc.los(T, src))
        got = unl[i][T.ls]
        assert np.max(np.abs(got[:, 0] / icl[:, 0] - 1)) < 1e-5
        assert np.max(np.abs(got[:, 1] / icl[:, 1] - 1)) < 1e-5
        assert np.max(np.abs(got[:, 3] - icl[:, 2]) / np.sqrt(icl[:, 0] * icl[:, 1])) < 1e-5


def test_lensed_massive_lmax2500():
    p = fiducial(2500, lensing=True, mnu=0.06, num_massive_neutrinos=1)
    T, allc, lensed = oracle_spectra(p)
    unl, lens, pot, lml = gpu_spectra([p], p.max_l)
    n = lensed.shape[0] - 1
    assert lml[0] == n
    check4(unl[0], as_tebt(allc), 2, p.max_l, bb=False)
    check4(lens[0], lensed, 2, n)


def test_transfer_kmax10():
    p = fiducial(2500, mnu=0.06, num_massive_neutrinos=1)
    p.want_cls, p.want_transfer, p.transfer_high_precision = 0, 1, 1
    p.transfer_kmax = 10 * p.H0 / 100
    p.num_transfer_redshifts = 1
    p.transfer_redshifts[0] = 0.0
    T = _lib.Tables(p)
    ref = orc.evolve_transfer(T)
    rs8, _ = orc.sigma8(T, ref)
    lib = _lib.load()
    tr = np.zeros((1, 1, 4096, 13), dtype=np.float32)
    nq = np.zeros(1, dtype=np.int32)
    s8 = np.zeros(1)
    st = np.zeros(1, dtype=np.int32)
    _lib.check(lib.cambgpu_get_transfer_batch(C.byref(p), 1, 4096, tr.ctypes.data_as(C.POINTER(C.c_float)),
                                              _lib.iptr(nq), _lib.dptr(s8), None, _lib.iptr(st)))
    assert nq[0] == T.view.nk
    got = tr[0, :, : nq[0]]
    peak = np.max(np.abs(ref), axis=1, keepdims=True)
    assert np.max(np.abs(got - ref) / np.where(peak > 0, peak, 1)) < 1e-5
    assert abs(s8[0] / rs8[0] - 1) < 1e-9


def test_lensed_massive_lmax2500_lens_potential_accuracy_4():
    """The same cosmology at the reference's automatic lens_potential_accuracy for lmax 2500
    (4: max_eta_k = 72000, so source modes to k ~ 5 /Mpc and Bessel arguments to 72000;
    linear lensing): sources of the highest-k modes and the C_l against the oracle."""
    p = fiducial(2500, lensing=True, mnu=0.06, num_massive_neutrinos=1)
    p.max_eta_k = 72000.0
    T, allc, lensed = oracle_spectra(p)
    assert T.view.nk > 250 and T.view.num_xx > 100000
    src = orc.evolve_sources(T)
    g = T.evolve_sources_gpu()
    assert rel_peak(g[..., -40:], src[..., -40:], axis=0) < 1e-6  # the 40 highest-k modes
    unl, lens, pot, lml = gpu_spectra([p], p.max_l)
    n = lensed.shape[0] - 1
    assert lml[0] == n
    check4(unl[0], as_tebt(allc), 2, p.max_l, bb=False)
    check4(lens[0], lensed, 2, n)
