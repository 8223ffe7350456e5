"""GPU parity under the reference's accuracy and model knobs (CAMBparams / AccuracyParams,
fortran/model.f90:27-209): one lensed 0.06 eV cosmology at lmax 1000 (+200 margin) per
setting, through cambgpu_get_spectra_batch in the FP64 form, against the oracle run on
the same tables -- unlensed C_l at every l and lensed C_l to the lensed lmax within 1e-5
(TE against sqrt(TT EE)), the lensing potential within 1e-5.  The settings move the
grids (k, q, time, l sampling), the hierarchy sizes, the stepper tolerance, the
switch times, the Limber and lensing ranges and the reionization history."""
import numpy as np
import pytest

from camb_gb300 import _lib
from oracle import oracle as orc
from tests.cosmologies import fiducial
from tests.test_gpu_lensing import as_tebt, check4, gpu_spectra

pytestmark = pytest.mark.gpu

SETTINGS = {
    "AccuracyBoost 2": dict(AccuracyBoost=2.0),
    "lAccuracyBoost 2, lSampleBoost 2": dict(lAccuracyBoost=2.0, lSampleBoost=2.0),
    "lAccuracyBoost 3 (photon hierarchy to l = 192)": dict(lAccuracyBoost=3.0),
    "k and time sampling boosts 1.5": dict(SourcekAccuracyBoost=1.5, IntkAccuracyBoost=1.5, TimeStepBoost=1.5),
    "tolerance, switch, Bessel, Limber boosts": dict(IntTolBoost=2.0, TimeSwitchBoost=1.5, BessIntBoost=1.5,
                                                     LimberBoost=1.5),
    "accurate_reionization off, accurate_polarization off": dict(accurate_reionization=0, accurate_polarization=0),
    "LensingBoost 2, Alens 0.7": dict(LensingBoost=2.0, Alens=0.7),
    "reionization at z = 8 (no optical depth)": dict(reion_use_optical_depth=0, reion_redshift=8.0),
    "YHe 0.25, TCMB 2.7, N_eff 3.3": dict(YHe=0.25, TCMB=2.7, nnu=3.3),
}


@pytest.fixture(autouse=True)
def fp64_form():
    lib = _lib.load()
    old = lib.cambgpu_get_precision()
    _lib.check(lib.cambgpu_set_precision(0))
    yield
    lib.cambgpu_set_precision(old)


@pytest.mark.parametrize("name", list(SETTINGS))
def test_setting_against_the_oracle(name):
    p = fiducial(1000, lensing=True, mnu=0.06, num_massive_neutrinos=1, **SETTINGS[name])
    T = _lib.Tables(p)
    icl = orc.cls(T, orc.los(T, orc.evolve_sources(T)))
    allc = orc.interpolate_cls(T.ls, icl, T.view.cl_template_scale)
    lensed = orc.lens_cls(allc[:, :4], T.ls, p.max_l, lens_accuracy_boost=T.view.lens_accuracy_boost)
    unl, lens, pot, lml = gpu_spectra([p], p.max_l)
    n = lensed.shape[0] - 1
    assert lml[0] == n
    check4(unl[0], as_tebt(allc), 2, p.max_l, bb=False)
    check4(lens[0], lensed, 2, n)
    ell = np.arange(2, p.max_l + 1, dtype=np.float64)
    pp = allc[2:, 3] * ((ell + 1) / ell) ** 2 / (2 * np.pi)  # the output's (L(L+1))^2 C_L/2pi
    assert np.max(np.abs(pot[0][2:, 0] / pp - 1)) < 1e-5


def test_raised_l_accuracy_on_the_thread_per_mode_kernel():
    """A batch at lAccuracyBoost 1.5 (photon hierarchies to l = 96) on the thread-per-mode
    kernel of large batches (team 7, static stride): C_l of three members against the
    oracle within 1e-5."""
    from tests.cosmologies import draws
    ps = draws(6, seed=55, lmax=1000, mnu_max=0.1)
    for p in ps:
        p.lAccuracyBoost = 1.5
    lib = _lib.load()
    _lib.check(lib.cambgpu_set_ode_team(7))
    _lib.check(lib.cambgpu_set_ode_schedule(1))
    try:
        unl, _, _, _ = gpu_spectra(ps, 1000)
    finally:
        lib.cambgpu_set_ode_team(0)
        lib.cambgpu_set_ode_schedule(-1)
    for i in (0, 2, 5):
        T = _lib.Tables(ps[i])
        icl = orc.cls(T, orc.los(T, orc.evolve_sources(T)))
        got = unl[i][T.ls]
        assert np.max(np.abs(got[:, 0] / icl[:, 0] - 1)) < 1e-5
        assert np.max(np.abs(got[:, 1] / icl[:, 1] - 1)) < 1e-5
        assert np.max(np.abs(got[:, 3] - icl[:, 2]) / np.sqrt(icl[:, 0] * icl[:, 1])) < 1e-5
