"""power_spectra_from_transfer: new primordial power applied to transfer functions kept on
the device gives the same spectra as evolving from scratch with that power (the
reference's camb.get_transfer_functions + CAMBdata.power_spectra_from_transfer)."""
import numpy as np
import pytest

from camb_gb300 import model, results

pytestmark = pytest.mark.gpu

BASE = dict(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.06, tau=0.06, lmax=800)


def test_power_spectra_from_transfer_matches_direct_run():
    tr = results.get_transfer_functions(model.set_params(As=2.1e-9, ns=0.965, **BASE))
    before = tr.get_lensed_scalar_cls()
    tr.power_spectra_from_transfer(model.InitialPowerLaw().set_params(As=2.4e-9, ns=0.95, nrun=0.01))
    cp = model.set_params(As=2.4e-9, ns=0.95, nrun=0.01, **BASE)
    direct = results.get_results(cp)
    for get in ("get_unlensed_scalar_cls", "get_lensed_scalar_cls", "get_lens_potential_cls"):
        a, b = getattr(tr, get)(), getattr(direct, get)()
        assert a.shape == b.shape
        assert np.allclose(a, b, rtol=1e-12, atol=0)
    assert not np.allclose(before, tr.get_lensed_scalar_cls(), rtol=1e-3, atol=0)


def test_batch_transfer_reuse_per_member():
    ps = [model.set_params(As=2.1e-9, ns=0.965, **dict(BASE, H0=h)) for h in (66.0, 68.0, 70.0)]
    trs = results.get_transfer_functions_batch(ps)
    trs[1].power_spectra_from_transfer(model.InitialPowerLaw().set_params(As=1.9e-9, ns=0.97))
    direct = results.get_results(model.set_params(As=1.9e-9, ns=0.97, **dict(BASE, H0=68.0)))
    assert np.allclose(trs[1].get_unlensed_scalar_cls(), direct.get_unlensed_scalar_cls(), rtol=1e-12, atol=0)
    other = results.get_results(ps[0])
    assert np.allclose(trs[0].get_unlensed_scalar_cls(), other.get_unlensed_scalar_cls(), rtol=1e-12, atol=0)


def test_stale_transfer_functions_refuse():
    tr = results.get_transfer_functions(model.set_params(As=2.1e-9, ns=0.965, **BASE))
    results.get_transfer_functions(model.set_params(As=2.1e-9, ns=0.965, **dict(BASE, H0=70.0)))
    with pytest.raises(Exception):
        tr.power_spectra_from_transfer(model.InitialPowerLaw().set_params(As=2.0e-9))
