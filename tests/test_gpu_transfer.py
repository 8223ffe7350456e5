"""GPU matter transfer functions (cambgpu_get_transfer_batch) against the oracle on the
same inputs, and the reference's sigma8 / f sigma8 known answers through the GPU path.
Tolerance: each transfer variable within 1e-5 of its peak over k (single-precision
storage, as the reference), sigma8 within 1e-6 relative of the oracle."""
import copy
import ctypes as C

import numpy as np
import pytest

from camb_gb300 import _lib
from oracle import oracle as orc
from tests.cosmologies import sigma8_known_answer

pytestmark = pytest.mark.gpu


def gpu_transfer(ps, nq_max=2048):
    lib = _lib.load()
    n = len(ps)
    nz = ps[0].num_transfer_redshifts
    arr = (_lib.CambGpuParams * n)(*ps)
    tr = np.zeros((n, nz, nq_max, 13), dtype=np.float32)
    nq = np.zeros(n, dtype=np.int32)
    s8 = np.zeros((n, nz))
    sv = np.zeros((n, nz))
    st = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_transfer_batch(arr, n, nq_max, tr.ctypes.data_as(C.POINTER(C.c_float)),
                                              _lib.iptr(nq), _lib.dptr(s8), _lib.dptr(sv), _lib.iptr(st)))
    assert not st.any()
    return tr, nq, s8, sv


@pytest.mark.parametrize("team", [0, 6, 2])
def test_transfer_functions_match_oracle_and_known_answers(team):
    """Autotuned kernel choice, warp per mode (shared-memory rows), thread per mode."""
    p, g = sigma8_known_answer()
    T = _lib.Tables(p)
    ref = orc.evolve_transfer(T)
    rs8, rsv = orc.sigma8(T, ref)
    lib = _lib.load()
    _lib.check(lib.cambgpu_set_ode_team(team))
    try:
        tr, nq, s8, sv = gpu_transfer([p])
    finally:
        lib.cambgpu_set_ode_team(0)
    assert nq[0] == T.view.nk
    got = tr[0, :, : nq[0]]
    peak = np.max(np.abs(ref), axis=1, keepdims=True)
    assert np.max(np.abs(got - ref) / np.where(peak > 0, peak, 1)) < 1e-5
    assert np.max(np.abs(s8[0] / rs8 - 1)) < 1e-6
    assert np.max(np.abs(sv[0] / rsv - 1)) < 1e-6
    fs8 = sv[0] / s8[0]
    for got_v, key in [(s8[0][0], "s8_z3.1"), (s8[0][2], "s8_z0"), (fs8[0], "fs8_z3.1"), (fs8[2], "fs8_z0")]:
        want, places = g[key]
        assert round(abs(got_v - want), places) == 0, (key, got_v, want)


def test_transfer_batch_of_masses():
    ps = []
    for m in (0.0, 0.06, 0.2):
        p, _ = sigma8_known_answer()
        p.mnu = m
        ps.append(p)
    tr, nq, s8, sv = gpu_transfer(ps)
    for i, p in enumerate(ps):
        T = _lib.Tables(p)
        ref = orc.evolve_transfer(T)
        rs8, _ = orc.sigma8(T, ref)
        assert np.max(np.abs(s8[i] / rs8 - 1)) < 1e-6
    # heavier neutrinos suppress the growth of structure
    assert s8[0][2] > s8[1][2] > s8[2][2]


def test_python_surface_sigma8():
    from camb_gb300 import model, results
    cp = model.set_params(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.07, As=2e-9, ns=0.965)
    cp.Reion.set_zrei(10)
    cp.WantCls = False
    cp.set_matter_power(redshifts=[0.0, 0.17, 3.1], kmax=1.2)
    r = results.get_results(cp)
    s8 = r.get_sigma8()
    assert abs(s8[0] - 0.24686) < 5e-4 and abs(s8[2] - 0.80044) < 5e-4
    assert abs(r.get_fsigma8()[2] - 0.424712) < 5e-4
    kh, z, pk = r.get_linear_matter_power_spectrum()
    assert list(z) == [0.0, 0.17, 3.1] and pk.shape == (3, len(kh))
    assert np.all(pk > 0) and pk[0].max() > pk[2].max()
    # the reference's P(k) known answers (camb_test.py testPowers, places=2)
    _, _, pks = r.get_matter_power_spectrum(1e-4, 1, 20)
    assert round(abs(pks[-1][-3] - 51.924), 2) == 0 and round(abs(pk[-2][-4] - 56.454), 2) == 0


def combined_known_answer():
    """testPowers as the reference runs it: the CMB on (lmax 2500, max_eta_k 5000) with
    high-precision transfer functions at z = 3.1, 0.17, 0."""
    p, g = sigma8_known_answer()
    p.want_cls = 1
    p.max_l, p.max_eta_k = 2500, 5000
    return p, g


def test_cmb_with_transfers_match_the_oracle():
    """A run that wants the CMB and transfer functions.  Transfer half on the GPU (the source
    grid plus the transfer grid above it; source modes stopping at every source time)
    against the oracle's single evolution of the whole run (CalcScalarSources with the
    transfer stops, TransferOut above): each variable within 1e-5 of its peak over k,
    sigma8 within 1e-6, and the known answers.  CMB half on the GPU (source modes at the
    /100 tolerance, kept to the last transfer time, no transfer stops) against the oracle's
    same form on the same tables: sources within 1e-6 of their peak."""
    p, g = combined_known_answer()
    T = _lib.Tables(p)
    t = T.transfer_view()
    src, ref = orc.evolve_combined(T)
    rs8, rsv = orc.sigma8(t, ref)
    tr, nq, s8, sv = gpu_transfer([p])
    assert nq[0] == t.nk and t.transfer_source_modes == T.view.nk
    got = tr[0, :, : nq[0]]
    peak = np.max(np.abs(ref), axis=1, keepdims=True)
    assert np.max(np.abs(got - ref) / np.where(peak > 0, peak, 1)) < 1e-5
    assert np.max(np.abs(s8[0] / rs8 - 1)) < 1e-6
    assert np.max(np.abs(sv[0] / rsv - 1)) < 1e-6
    fs8 = sv[0] / s8[0]
    for got_v, key in [(s8[0][0], "s8_z3.1"), (s8[0][2], "s8_z0"), (fs8[0], "fs8_z3.1"), (fs8[2], "fs8_z0")]:
        want, places = g[key]
        assert round(abs(got_v - want), places) == 0, (key, got_v, want)
    gs = T.evolve_sources_gpu()
    cpu = orc.evolve_sources(T)  # the same form: no transfer stops
    num = np.max(np.abs(gs - cpu), axis=0)
    den = np.max(np.abs(cpu), axis=0)
    m = den > 0
    assert np.max(num[m] / den[m]) < 1e-6


def both_in_one_launch(ps, lmax, nq_max=2048):
    lib = _lib.load()
    n = len(ps)
    nz = ps[0].num_transfer_redshifts
    arr = (_lib.CambGpuParams * n)(*ps)
    cls = np.zeros((n, lmax + 1, 4))
    tr = np.zeros((n, nz, nq_max, 13), dtype=np.float32)
    nq = np.zeros(n, dtype=np.int32)
    s8 = np.zeros((n, nz))
    sv = np.zeros((n, nz))
    st = np.zeros(n, dtype=np.int32)
    lml = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_results_with_transfers(arr, n, lmax, _lib.dptr(cls), None, None, _lib.iptr(lml), nq_max,
                                                      tr.ctypes.data_as(C.POINTER(C.c_float)), _lib.iptr(nq),
                                                      _lib.dptr(s8), _lib.dptr(sv), _lib.iptr(st)))
    assert not st.any()
    return cls, tr, nq, s8, sv


@pytest.mark.parametrize("zs", [(3.1, 0.17, 0.0), (3.1, 1.0)])
def test_single_launch_is_the_single_evolution(zs):
    """cambgpu_get_results_with_transfers: one transfer-path launch stores the source modes'
    CMB sources at the source times and their transfer variables at the transfer times.
    Against the oracle's single evolution of the run: transfer variables within 1e-5 of
    their peak, sigma8 within 1e-6, and the C_l of its sources (the FP64 projection) within
    1e-5 at the sampled l -- also when the last transfer time is before today (the source
    modes then keep storing sources to the late-time cut)."""
    p, _ = combined_known_answer()
    p.num_transfer_redshifts = len(zs)
    for i, z in enumerate(zs):
        p.transfer_redshifts[i] = z
    p.max_l, p.max_eta_k = 1500, 3750
    T = _lib.Tables(p)
    t = T.transfer_view()
    src, ref = orc.evolve_combined(T)
    icl = orc.cls(T, orc.los(T, src))
    rs8, _ = orc.sigma8(t, ref)
    cls, tr, nq, s8, _ = both_in_one_launch([p], 1500)
    assert nq[0] == t.nk
    got = tr[0, :, : nq[0]]
    peak = np.max(np.abs(ref), axis=1, keepdims=True)
    assert np.max(np.abs(got - ref) / np.where(peak > 0, peak, 1)) < 1e-5
    assert np.max(np.abs(s8[0] / rs8 - 1)) < 1e-6
    g = cls[0][T.ls]
    assert np.max(np.abs(g[:, 0] / icl[:, 0] - 1)) < 1e-5
    assert np.max(np.abs(g[:, 1] / icl[:, 1] - 1)) < 1e-5
    assert np.max(np.abs(g[:, 3] - icl[:, 2]) / np.sqrt(icl[:, 0] * icl[:, 1])) < 1e-5


def test_single_launch_lensed():
    """The single launch with lensing on: the lensed C_l and the lensing potential of the
    CMB half match the two-call form (whose CMB half lacks only the transfer stops) to
    1e-6, and sigma8 is the transfer call's."""
    from camb_gb300 import model, results
    cp = model.set_params(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.06, As=2.1e-9, ns=0.965, lmax=1000)
    cp.set_matter_power(redshifts=[0.5, 0.0], kmax=1.0)
    one = results.get_results(cp)
    two = results._run([cp], 1000)[0]
    a, b = one.get_lensed_scalar_cls(1000)[2:], two.get_lensed_scalar_cls(1000)[2:]
    assert np.max(np.abs(a[:, :2] / b[:, :2] - 1)) < 1e-6
    pa, pb = one.get_lens_potential_cls(1000)[2:, 0], two.get_lens_potential_cls(1000)[2:, 0]
    assert np.max(np.abs(pa / pb - 1)) < 1e-6
    _, _, s8, _ = gpu_transfer([cp.to_struct()])
    assert np.array_equal(one.get_sigma8(), s8[0])


def test_cmb_with_transfers_ending_before_today():
    """Transfer redshifts 3.1 and 1 only: the CMB half's modes keep evolving to z = 1 and
    then take the late-time cut (src_keep_tau below tau0), the transfer half's source modes
    stop at the source times up to z = 1; both against the oracle on the same tables
    (sources within 1e-6 of their peak; transfers within 1e-5 of theirs)."""
    p, _ = combined_known_answer()
    p.num_transfer_redshifts = 2
    p.transfer_redshifts[0], p.transfer_redshifts[1] = 3.1, 1.0
    p.max_l, p.max_eta_k = 1500, 3750
    T = _lib.Tables(p)
    t = T.transfer_view()
    assert T.view.src_keep_tau < 0.9 * T.view.tau0
    _, ref = orc.evolve_combined(T)
    tr, nq, _, _ = gpu_transfer([p])
    got = tr[0, :, : nq[0]]
    peak = np.max(np.abs(ref), axis=1, keepdims=True)
    assert nq[0] == t.nk
    assert np.max(np.abs(got - ref) / np.where(peak > 0, peak, 1)) < 1e-5
    cpu = orc.evolve_sources(T)
    gs = T.evolve_sources_gpu()
    num = np.max(np.abs(gs - cpu), axis=0)
    den = np.max(np.abs(cpu), axis=0)
    m = den > 0
    assert np.max(num[m] / den[m]) < 1e-6


def test_cmb_with_transfers_batch_of_masses():
    """Three such runs in one transfer launch (each cosmology its own source grid, so its
    own number of modes that stop at the source times), each against the oracle's single
    evolution of its run."""
    ps = []
    for m in (0.0, 0.06, 0.2):
        p, _ = combined_known_answer()
        p.mnu = m
        p.max_l, p.max_eta_k = 1200, 3000
        ps.append(p)
    tr, nq, s8, _ = gpu_transfer(ps)
    for i, p in enumerate(ps):
        T = _lib.Tables(p)
        t = T.transfer_view()
        _, ref = orc.evolve_combined(T)
        assert nq[i] == t.nk
        got = tr[i, :, : nq[i]]
        peak = np.max(np.abs(ref), axis=1, keepdims=True)
        assert np.max(np.abs(got - ref) / np.where(peak > 0, peak, 1)) < 1e-5
        rs8, _ = orc.sigma8(t, ref)
        assert np.max(np.abs(s8[i] / rs8 - 1)) < 1e-6
    assert s8[0][2] > s8[1][2] > s8[2][2]


def test_python_surface_cmb_and_matter_power_together():
    """set_matter_power with the CMB on (the reference's usual call): one result object with
    the C_l and the transfer functions of the single launch, equal to that C-ABI call on
    the same parameters; the two-call form (CMB half without the transfer stops) agrees to
    1e-7 in the C_l and exactly in sigma8."""
    from camb_gb300 import model, results
    cp = model.set_params(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.06, As=2.1e-9, ns=0.965, lmax=800,
                          DoLensing=False)
    cp.set_matter_power(redshifts=[0.0], kmax=1.0)
    both = results.get_results(cp)
    cls, _, _, s8, _ = both_in_one_launch([cp.to_struct()], 800)
    assert np.array_equal(both._cls, cls[0]) and both.get_sigma8()[0] == s8[0][0]
    two = results._run([cp], 800)[0].get_unlensed_scalar_cls(800)
    one = both.get_unlensed_scalar_cls(800)
    assert np.max(np.abs(one[2:, :2] / two[2:, :2] - 1)) < 1e-7
    _, _, s8t, _ = gpu_transfer([cp.to_struct()])
    assert both.get_sigma8()[0] == s8t[0][0]
    assert 0.7 < both.get_sigma8()[0] < 0.9


def test_top_level_matter_power_interpolator():
    """camb.get_matter_power_interpolator(params): transfer functions at the default 100
    redshifts (0-10) to kmax 10 /Mpc on the GPU; at z = 0 the spline agrees with the
    log-grid power of a single-redshift run within 2e-3, and P falls with z."""
    import camb_gb300 as camb
    from camb_gb300 import model
    cp = model.set_params(H0=67.5, ombh2=0.022, omch2=0.122, mnu=0.06, As=2e-9, ns=0.965, lmax=1000)
    PK, zs, kh = camb.get_matter_power_interpolator(cp, nonlinear=False, return_z_k=True)
    assert len(zs) == 100 and zs[0] == 0.0 and abs(zs[-1] - 10.0) < 1e-9
    one = copy.deepcopy(cp)
    one.set_matter_power(redshifts=[0.0], kmax=10.0)
    one.WantCls = False
    khs, _, pk = camb.get_results(one).get_matter_power_spectrum(1e-3, 5.0, 40)
    np.testing.assert_allclose(PK.P(0.0, khs), pk[0], rtol=2e-3)
    p = PK.P(np.array([0.0, 1.0, 5.0]), np.array([0.2]))[:, 0]
    assert p[0] > p[1] > p[2] > 0
