"""GPU parity with massive neutrinos: the momentum-binned massive-neutrino hierarchy,
its switches (relativistic bins, non-relativistic truncation, fluid approximation) and
the repacking of the state vector at each switch, against the oracle on the same
inputs.  Tolerances as for the massless path: sources within 1e-6 of their peak per
k-mode, Delta_l(k) within 1e-6 relative, C_l within 1e-5 relative."""
import ctypes as C

import numpy as np
import pytest

from camb_gb300 import _lib
from oracle import oracle as orc
from tests.cosmologies import draws, fiducial, planck2018

pytestmark = pytest.mark.gpu


def rel_peak(a, b, axis):
    num = np.max(np.abs(a - b), axis=axis)
    den = np.max(np.abs(b), axis=axis)
    m = den > 0
    return float(np.max(num[m] / den[m])) if np.any(m) else 0.0


def check_cls(got, icl, tol=1e-5):
    assert np.max(np.abs(got[:, 0] / icl[:, 0] - 1)) < tol
    assert np.max(np.abs(got[:, 1] / icl[:, 1] - 1)) < tol
    assert np.max(np.abs(got[:, 3] - icl[:, 2]) / np.sqrt(icl[:, 0] * icl[:, 1])) < tol


@pytest.fixture(scope="module")
def planck():
    T = _lib.Tables(planck2018(1000))
    assert T.view.nu_eig == 1
    src = orc.evolve_sources(T)
    return T, src


def with_team(team, f):
    lib = _lib.load()
    _lib.check(lib.cambgpu_set_ode_team(team))
    try:
        return f()
    finally:
        lib.cambgpu_set_ode_team(0)


@pytest.mark.parametrize("team", [0, 6, 2, 7])
def test_sources_parity_006ev(planck, team):
    """Autotuned choice, warp per mode (shared-memory rows), thread per mode."""
    T, src = planck
    g = with_team(team, T.evolve_sources_gpu)
    assert rel_peak(g, src, axis=0) < 1e-6


def test_end_to_end_cls_006ev(planck):
    T, src = planck
    icl = orc.cls(T, orc.los(T, src))
    cls = np.zeros((1001, 4))
    p = planck2018(1000)
    _lib.check(_lib.load().cambgpu_get_results(C.byref(p), 1000, _lib.dptr(cls)))
    check_cls(cls[T.ls], icl)


@pytest.mark.parametrize("team", [0, 6])
@pytest.mark.parametrize("mnu", [0.2, 0.6])
def test_sources_parity_heavier(mnu, team):
    """Heavier eigenstates: more momentum bins, longer hierarchies, earlier switches."""
    T = _lib.Tables(fiducial(600, mnu=mnu, num_massive_neutrinos=1))
    src = orc.evolve_sources(T)
    g = with_team(team, T.evolve_sources_gpu)
    assert rel_peak(g, src, axis=0) < 1e-6


def test_batch_mixed_massive_and_massless():
    """A batch of draws with mnu uniform in [0, 0.2] eV plus one massless cosmology: the
    register-resident warp kernel (32 lanes) is massless-only, so a request for it runs
    the batch on the shared-memory warp-per-mode kernel."""
    ps = draws(3, seed=11, lmax=600, mnu_max=0.2) + [fiducial(600)]
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    cls = np.zeros((len(ps), 601, 4))
    st = np.zeros(len(ps), dtype=np.int32)
    lib = _lib.load()
    _lib.check(lib.cambgpu_set_ode_team(32))
    try:
        _lib.check(lib.cambgpu_get_results_batch(arr, len(ps), 600, _lib.dptr(cls), _lib.iptr(st)))
    finally:
        lib.cambgpu_set_ode_team(0)
    assert not st.any()
    for i, p in enumerate(ps):
        T = _lib.Tables(p)
        icl = orc.cls(T, orc.los(T, orc.evolve_sources(T)))
        check_cls(cls[i][T.ls], icl)
