"""The CAMBdata spectrum getters on CPU (no device call: the results object is built from
arrays): unit and raw-C_l conversions as in the reference's results.py:417-444, the
spectra dictionary of get_cmb_power_spectra, and the text file of
save_cmb_power_spectra (results.py:62-82, 459-472)."""
import numpy as np
import pytest

from camb_gb300 import model, results


@pytest.fixture()
def data():
    p = model.set_params(lmax=60, DoLensing=True)
    rng = np.random.default_rng(0)
    n = p.max_l + 1
    unl = np.abs(rng.normal(size=(n, 4))) * 1e-10
    lensed = unl * 1.01
    pot = np.abs(rng.normal(size=(n, 3))) * 1e-8
    return p, results.CAMBdata(p, unl, lensed=lensed, lens_potential=pot, lmax_lensed=60), unl, lensed, pot


def test_raw_cl_and_units_follow_the_reference(data):
    p, d, unl, lensed, pot = data
    ell = np.arange(1, 61, dtype=np.float64)
    llp1 = ell * (ell + 1)
    raw = d.get_lensed_scalar_cls(CMB_unit="muK", raw_cl=True)
    u = p.TCMB * 1e6
    np.testing.assert_allclose(raw[1:], lensed[1:61] / (llp1 / (2 * np.pi))[:, None] * u ** 2, rtol=1e-14)
    assert np.all(raw[0] == lensed[0] * u ** 2)
    pp = d.get_lens_potential_cls(lmax=60, CMB_unit="K", raw_cl=True)
    np.testing.assert_allclose(pp[1:, 0], pot[1:61, 0] / (llp1 ** 2 / (2 * np.pi)), rtol=1e-14)
    np.testing.assert_allclose(pp[1:, 1:], pot[1:61, 1:] / (llp1 ** 1.5 / (2 * np.pi))[:, None] * p.TCMB,
                               rtol=1e-14)
    with pytest.raises(ValueError):
        d.get_unlensed_scalar_cls(CMB_unit="mK")


def test_power_spectra_dictionary(data):
    p, d, unl, lensed, pot = data
    P = d.get_cmb_power_spectra(CMB_unit="muK")
    assert set(P) == {"total", "unlensed_scalar", "unlensed_total", "lensed_scalar", "tensor", "lens_potential"}
    for v in P.values():
        assert v.shape[0] == 61
    np.testing.assert_array_equal(P["total"], P["lensed_scalar"])
    assert not P["tensor"].any()


def test_save_cmb_power_spectra_text_file(data, tmp_path):
    p, d, unl, lensed, pot = data
    fn = tmp_path / "cls.dat"
    d.save_cmb_power_spectra(str(fn))
    with open(fn) as f:
        head = f.readline()
    assert head.split() == ["#", "L", "TT", "EE", "BB", "TE", "PP", "PT", "PE"]
    arr = np.loadtxt(fn)
    assert arr.shape == (61, 8)
    assert np.array_equal(arr[:, 0], np.arange(61))
    np.testing.assert_allclose(arr[:, 1:5], d.get_total_cls(CMB_unit="muK"), rtol=1e-7)
    np.testing.assert_allclose(arr[:, 5:], d.get_lens_potential_cls(60, CMB_unit="muK"), rtol=1e-7)


def test_shared_grid_api_checks_its_arguments_before_any_device_call():
    p = model.set_params(lmax=100)
    with pytest.raises(model.CAMBError):
        results.get_results_batch_shared([p], projection="fp16")
    t = model.set_params(lmax=100)
    t.WantTransfer = True
    with pytest.raises(model.CAMBError):
        results.get_results_batch_shared([t])


def test_set_accuracy_and_dark_energy_follow_the_reference():
    """set_accuracy sets the three overall knobs (model.py set_accuracy); set_dark_energy()
    with its defaults is accepted (the reference's cosmological constant) and any other
    equation of state raises, as do the accuracy options this path does not build."""
    p = model.set_params(lmax=100)
    assert p.set_accuracy(AccuracyBoost=2, lSampleBoost=1.5, lAccuracyBoost=3) is p
    assert (p.Accuracy.AccuracyBoost, p.Accuracy.lSampleBoost, p.Accuracy.lAccuracyBoost) == (2, 1.5, 3)
    s = p.to_struct()
    assert (s.AccuracyBoost, s.lSampleBoost, s.lAccuracyBoost) == (2, 1.5, 3)
    assert p.set_dark_energy() is p
    for bad in (dict(w=-0.9), dict(wa=0.1), dict(use_tabulated_w=True)):
        with pytest.raises(model.CAMBError):
            p.set_dark_energy(**bad)
    with pytest.raises(model.CAMBError):
        p.set_accuracy(DoLateRadTruncation=False)


def test_set_params_routes_keywords_like_the_reference():
    """camb.set_params routing (camb.py:200-238): accuracy and dark-energy keywords go to
    their setters, dotted names reach sub-objects, and an unknown name raises instead of
    being stored and ignored."""
    p = model.set_params(lmax=100, AccuracyBoost=1.5, w=-1.0, **{"Accuracy.IntTolBoost": 2.0})
    assert p.Accuracy.AccuracyBoost == 1.5 and p.Accuracy.IntTolBoost == 2.0
    with pytest.raises(model.CAMBError):
        model.set_params(lmax=100, w=-0.9)
    with pytest.raises(model.CAMBError):
        model.set_params(lmax=100, not_a_parameter=1)
