"""Host construction of grids shared by a batch (cambgpu_tables_share_grids), the input of
the tensor-core projection: every member's time steps are tau0 - chi_n on one comoving-
distance grid, whose spacing follows the finest native spacing of any member at each chi,
and the members share one source k grid, one integration q grid and one Bessel table.
The C_l on shared grids differ from those on each member's native grids by the
discretization error of the default accuracy itself (measured here with the oracle)."""
import ctypes as C

import numpy as np

from camb_gb300 import _lib
from camb_gb300.workload import batch_draws
from oracle import oracle as orc


def shared_tables(ps):
    lib = _lib.load()
    ts = [_lib.Tables(p) for p in ps]
    arr = (C.c_void_p * len(ts))(*[t.handle for t in ts])
    nchi = C.c_int()
    _lib.check(lib.cambgpu_tables_share_grids(arr, len(ts), C.byref(nchi)))
    for t in ts:
        _lib.check(lib.cambgpu_tables_view(t.handle, C.byref(t.view)))
    return ts, nchi.value


def test_shared_grid_structure():
    ps = batch_draws(4, 1000, seed=11)
    nat = [_lib.Tables(p) for p in ps]
    ts, nchi = shared_tables(ps)
    v0 = ts[0].view
    for t, n in zip(ts, nat):
        v = t.view
        assert v.nk == v0.nk and v.nq == v0.nq and v.nl == v0.nl and v.num_xx == v0.num_xx
        assert np.array_equal(t.q_evolve, ts[0].q_evolve) and np.array_equal(t.q_int, ts[0].q_int)
        tau = t.tau_points
        assert v.ntau <= nchi and tau[-1] == v.tau0 and np.all(np.diff(tau) > 0)
        chi = v.tau0 - tau
        # the shared grid is at least as fine as the member's native time steps where they overlap
        nt = n.tau_points
        lo, hi = np.searchsorted(tau, nt[0]), len(tau)
        step = np.diff(tau[lo:hi])
        native = np.interp(tau[lo:hi - 1], nt[:-1], np.diff(nt))
        assert np.all(step <= native * (1 + 1e-9))
    # every member's nodes are one grid in chi
    chi0 = ts[0].view.tau0 - ts[0].tau_points
    for t in ts[1:]:
        chi = t.view.tau0 - t.tau_points
        m = min(len(chi), len(chi0))
        np.testing.assert_allclose(chi[-m:], chi0[-m:], rtol=0, atol=1e-9 * t.view.tau0)


def test_shared_grid_shift_of_cls_is_the_discretization_error():
    """Oracle C_l (lmax 1000) of three draws on shared vs native grids: within 2e-3."""
    ps = batch_draws(3, 1000, seed=12)
    nat = [_lib.Tables(p) for p in ps]
    ts, _ = shared_tables(ps)
    for t, n in zip(ts, nat):
        cs = orc.cls(t, orc.los(t, orc.evolve_sources(t)))
        cn = orc.cls(n, orc.los(n, orc.evolve_sources(n)))
        assert np.max(np.abs(cs[:, 0] / cn[:, 0] - 1)) < 2e-3
        assert np.max(np.abs(cs[:, 1] / cn[:, 1] - 1)) < 2e-3


def test_shared_grid_extreme_members_lmax2500():
    """The members with the smallest and largest tau0 of 16 draws at lmax 2500: the shared
    q grid (from the median member) reaches Bessel arguments q chi beyond the largest
    member's own q_max tau0, so the shared Bessel table must extend past every member's
    own; C_l within 2e-3 of each member's native grids at every sampled l."""
    ps = batch_draws(16, 2500, seed=13)
    ts, _ = shared_tables(ps)
    tau0 = np.array([t.view.tau0 for t in ts])
    for i in (int(np.argmin(tau0)), int(np.argmax(tau0))):
        t, n = ts[i], _lib.Tables(ps[i])
        cs = orc.cls(t, orc.los(t, orc.evolve_sources(t)))
        cn = orc.cls(n, orc.los(n, orc.evolve_sources(n)))
        assert np.max(np.abs(cs[:, 0] / cn[:, 0] - 1)) < 2e-3
        assert np.max(np.abs(cs[:, 1] / cn[:, 1] - 1)) < 2e-3
