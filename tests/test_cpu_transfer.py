"""CPU tests of the matter-transfer restatement: the oracle's sigma8 and f sigma8 against
the reference's known answers (camb/tests/camb_test.py testPowers, places=3), which pins
the massive-neutrino ODE at the 1e-4 level; and the transfer k grid and mode set-up."""
import numpy as np
import pytest

from camb_gb300 import _lib
from oracle import oracle as orc
from tests.cosmologies import sigma8_known_answer


@pytest.fixture(scope="module")
def run():
    p, g = sigma8_known_answer()
    T = _lib.Tables(p)
    tr = orc.evolve_transfer(T)
    s8, sv = orc.sigma8(T, tr)
    return T, tr, s8, sv, g


def test_sigma8_known_answers(run):
    """The reference computes these with the CMB on (its transfer k grid then starts from
    the CMB source grid); here the transfer functions are computed alone on the transfer
    grid.  Agreement is 3e-5, well inside the reference's places=3."""
    _, _, s8, sv, g = run
    fs8 = sv / s8
    for got, key in [(s8[0], "s8_z3.1"), (s8[2], "s8_z0"), (fs8[0], "fs8_z3.1"), (fs8[2], "fs8_z0")]:
        want, places = g[key]
        assert round(abs(got - want), places) == 0, (key, got, want)
        assert abs(got - want) < 1e-4, (key, got, want)


def test_transfer_grid_and_outputs(run):
    T, tr, s8, _, _ = run
    v = T.view
    q = T.q_evolve
    assert v.transfer_only == 1 and v.num_transfer_times == 3
    assert np.all(np.diff(q) > 0) and q[0] == pytest.approx(5e-5) and q[-1] <= 1.2 * 1.05 * (1 + 1e-12)
    times = [v.transfer_times[i] for i in range(3)]
    assert times[0] < times[1] < times[2] and times[2] == pytest.approx(v.tau0, rel=1e-6)
    assert tr.dtype == np.float32 and tr.shape == (3, v.nk, 13)
    assert np.allclose(tr[0, :, 0] * v.hubble_h, q, rtol=1e-6)   # k/h column
    assert np.all(np.isfinite(tr))
    # growth: the total matter transfer grows from z = 3.1 to 0 on every scale
    assert np.all(tr[2, :, 6] > tr[0, :, 6])
    assert s8[0] < s8[1] < s8[2]


def combined_known_answer():
    """The testPowers cosmology as the reference runs it there: the CMB on (lmax 2500,
    max_eta_k 5000) with high-precision transfer functions at z = 3.1, 0.17, 0."""
    p, g = sigma8_known_answer()
    p.want_cls = 1
    p.max_l, p.max_eta_k = 2500, 5000
    return p, g


@pytest.fixture(scope="module")
def combined():
    p, g = combined_known_answer()
    T = _lib.Tables(p)
    src, tr = orc.evolve_combined(T)
    return T, src, tr, g


def test_cmb_with_transfers_tables(combined):
    """A run that wants the CMB and transfer functions: the CMB half carries the /100
    tolerance and the 20-per-e-fold source grid of high-precision transfers
    (cmbmain.f90:875-893, 1018-1021) and keeps its modes to the last transfer time; the
    transfer half is the source grid followed by the transfer grid above it (InitTransfer with
    WantCls, cmbmain.f90:681-699), its source modes flagged to stop at the source times."""
    T, _, _, _ = combined
    v, t = T.view, T.transfer_view()
    p0, _ = combined_known_answer()
    p0.want_transfer = 0
    T0 = _lib.Tables(p0)
    assert v.tol1 == pytest.approx(T0.view.tol1 / 100) and v.nk > T0.view.nk
    q = T.q_evolve
    qt = np.ctypeslib.as_array(t.q_evolve, shape=(t.nk,))
    assert t.transfer_only == 1 and t.want_cls == 1 and t.transfer_source_modes == v.nk
    assert np.array_equal(qt[: v.nk], q) and np.all(qt[v.nk:] > q[-1] + 1e-4) and np.all(np.diff(qt) > 0)
    assert v.src_keep_tau == t.transfer_times[t.num_transfer_times - 1]
    assert T0.view.src_keep_tau == -1 and T0.view.transfer_source_modes == 0
    with pytest.raises(_lib.CAMBError):
        T0.transfer_view()


def test_cmb_with_transfers_known_answers(combined):
    """testPowers is this run: the exact restatement of it (the source modes stopping at the
    transfer times inside CalcScalarSources, TransferOut above the source grid) meets the
    sigma8 and f sigma8 known answers to places=3 (and within 1e-4)."""
    T, _, tr, g = combined
    s8, sv = orc.sigma8(T.transfer_view(), tr)
    fs8 = sv / s8
    for got, key in [(s8[0], "s8_z3.1"), (s8[2], "s8_z0"), (fs8[0], "fs8_z3.1"), (fs8[2], "fs8_z0")]:
        want, places = g[key]
        assert round(abs(got - want), places) == 0, (key, got, want)
        assert abs(got - want) < 1e-4, (key, got, want)


def test_cmb_half_matches_the_single_evolution(combined):
    """The library's CMB half evolves the source modes without the transfer stops.  At the
    high-precision tolerance its sources differ from the reference's single evolution by
    under 1e-9 of each mode's peak (measured 4.8e-11) and the C_l by under 1e-10."""
    T, src, _, _ = combined
    src_h = orc.evolve_sources(T)
    peak = np.abs(src).max(axis=(0, 1), keepdims=True)
    assert np.max(np.abs(src_h - src) / np.maximum(peak, 1e-300)) < 1e-9
    cl = orc.cls(T, orc.los(T, src))
    cl_h = orc.cls(T, orc.los(T, src_h))
    assert np.max(np.abs(cl_h[:, :2] / cl[:, :2] - 1)) < 1e-10


def test_matter_power_known_answers():
    """get_matter_power_spectrum (the transfer functions splined in ln k,
    Transfer_GetMatterPowerD) and get_linear_matter_power_spectrum (the transfer grid) on
    the oracle's transfer functions against the reference's known answers
    (camb_test.py testPowers, places=2)."""
    import json
    import os
    from camb_gb300 import model, results
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))["matter_power"]
    cp = model.set_params(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.07, As=2e-9, ns=0.965)
    cp.Reion.set_zrei(10)
    cp.WantCls = False
    cp.set_matter_power(redshifts=[0.0, 0.17, 3.1], kmax=1.2)
    T = _lib.Tables(cp.to_struct())
    tr = orc.evolve_transfer(T)
    td = np.ascontiguousarray(tr.transpose(2, 1, 0))
    s8, sv = orc.sigma8(T, tr)
    r = results.CAMBdataMatter(cp, results.MatterTransferData(td, td[0, :, 0] * cp.H0 / 100, s8, sv))
    kh, z, pk = r.get_matter_power_spectrum(1e-4, 1, 20)
    assert list(z) == [0.0, 0.17, 3.1] and pk.shape == (3, 20)
    np.testing.assert_allclose(kh, np.logspace(-4, 0, 20), rtol=1e-12)
    kh2, _, pk2 = r.get_linear_matter_power_spectrum()
    for got, key in [(pk[g["splined"]["index"][0], g["splined"]["index"][1]], "splined"),
                     (pk2[g["unsplined"]["index"][0], g["unsplined"]["index"][1]], "unsplined")]:
        want, places = g[key]["value"]
        assert round(abs(got - want), places) == 0, (key, got, want)
    # at the transfer grid's own k the spline returns the unsplined values
    inner = slice(3, len(kh2) - 3)
    for zi in range(3):
        for j in range(inner.start, inner.stop, 7):
            _, _, one = r.get_matter_power_spectrum(kh2[j], kh2[j] * 1.5, 2)
            np.testing.assert_allclose(one[zi, 0], pk2[zi, j], rtol=1e-5)


def test_matter_power_known_answers_with_the_cmb_on():
    """The same P(k) known answers from the run testPowers actually makes (the CMB on, lmax
    2500): the exact restatement of that single evolution, on its transfer grid (the 20
    per e-fold source grid followed by the transfer grid above it)."""
    import json
    import os
    from camb_gb300 import model, results
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))["matter_power"]
    cp = model.set_params(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.07, As=2e-9, ns=0.965, lmax=2500,
                          DoLensing=False)
    cp.Reion.set_zrei(10)
    cp.set_matter_power(redshifts=[0.0, 0.17, 3.1], kmax=1.2)
    T = _lib.Tables(cp.to_struct())
    t = T.transfer_view()
    _, tr = orc.evolve_combined(T)
    td = np.ascontiguousarray(tr.transpose(2, 1, 0))
    s8, sv = orc.sigma8(t, tr)
    r = results.CAMBdataMatter(cp, results.MatterTransferData(td, td[0, :, 0] * cp.H0 / 100, s8, sv))
    _, _, pk = r.get_matter_power_spectrum(1e-4, 1, 20)
    _, _, pk2 = r.get_linear_matter_power_spectrum()
    for got, key in [(pk[g["splined"]["index"][0], g["splined"]["index"][1]], "splined"),
                     (pk2[g["unsplined"]["index"][0], g["unsplined"]["index"][1]], "unsplined")]:
        want, places = g[key]["value"]
        assert round(abs(got - want), places) == 0, (key, got, want)


def test_matter_power_interpolator():
    """get_matter_power_interpolator on the oracle's transfer functions: through the
    transfer-grid power at every node, within 2e-3 of the log-grid spline between nodes at
    the computed redshifts, monotone growth at intermediate z, a single-redshift run that
    refuses other z, and the power-law continuation to extrap_kmax."""
    from camb_gb300 import model, results
    cp = model.set_params(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.07, As=2e-9, ns=0.965)
    cp.Reion.set_zrei(10)
    cp.WantCls = False
    cp.set_matter_power(redshifts=[0.0, 0.17, 0.5, 1.0, 3.1], kmax=1.2)
    T = _lib.Tables(cp.to_struct())
    tr = orc.evolve_transfer(T)
    td = np.ascontiguousarray(tr.transpose(2, 1, 0))
    s8, sv = orc.sigma8(T, tr)
    r = results.CAMBdataMatter(cp, results.MatterTransferData(td, td[0, :, 0] * cp.H0 / 100, s8, sv))
    kh, z, pk = r.get_linear_matter_power_spectrum()
    PK = r.get_matter_power_interpolator(nonlinear=False)
    np.testing.assert_allclose(PK.P(z, kh), pk, rtol=1e-10)
    khs, _, pks = r.get_matter_power_spectrum(1e-3, 1.0, 50)
    np.testing.assert_allclose(PK.P(z, khs), pks, rtol=2e-3)
    mid = PK.P(np.array([0.3, 0.7]), np.array([0.1]))
    assert pk[1, np.searchsorted(kh, 0.1)] > mid[0, 0] > mid[1, 0] > pk[3, np.searchsorted(kh, 0.1)] * 0.9
    ext = r.get_matter_power_interpolator(nonlinear=False, extrap_kmax=10.0)
    assert ext.kmax == kh[-1] and np.isfinite(ext.P(0.0, 5.0))
    slope = np.log(pk[0, -1] / pk[0, -2]) / np.log(kh[-1] / kh[-2])
    np.testing.assert_allclose(np.log(ext.P(0.0, 10.0) / pk[0, -1]) / np.log(10.0 / kh[-1]), slope, rtol=1e-6)
    one = results.MatterPowerInterpolator([0.5], kh, pk[2:3])
    np.testing.assert_allclose(one.P(0.5, kh), pk[2], rtol=1e-10)
    with pytest.raises(_lib.CAMBError):
        one.P(0.0, 0.1)
