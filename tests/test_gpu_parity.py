"""GPU parity: the CUDA path through the C ABI against the CPU oracle on the same
inputs.  Tolerances: transfer functions Delta_l(k) within 1e-6 relative and C_l
within 1e-5 relative (the plain FP64 GPU form); sources per k-mode within 1e-6 of
their peak."""
import ctypes as C

import numpy as np
import pytest

from camb_gb300 import _lib
from oracle import oracle as orc
from tests.cosmologies import draws, fiducial

pytestmark = pytest.mark.gpu


def rel_peak(a, b, axis):
    """max |a-b| / max|b| along the reduced axis (entries whose peak is zero are skipped)."""
    num = np.max(np.abs(a - b), axis=axis)
    den = np.max(np.abs(b), axis=axis)
    m = den > 0
    return float(np.max(num[m] / den[m])) if np.any(m) else 0.0


@pytest.fixture(scope="module")
def fid():
    T = _lib.Tables(fiducial(1000))
    src = orc.evolve_sources(T)
    delta = orc.los(T, src)
    icl = orc.cls(T, delta)
    return T, src, delta, icl


def test_sources_parity(fid):
    T, src, _, _ = fid
    g = T.evolve_sources_gpu()
    assert g.shape == src.shape
    # per (source, k-mode): compare over time
    assert rel_peak(g, src, axis=0) < 1e-6


def test_los_parity_same_sources(fid):
    T, src, delta, _ = fid
    g = T.los_gpu(src)
    # Delta_l(k) relative 1e-6 where |Delta| > 1e-3 of its peak over l
    peak = np.max(np.abs(delta), axis=1, keepdims=True)
    m = np.abs(delta) > 1e-3 * peak
    err = np.abs(g - delta)[m] / np.abs(delta)[m]
    assert err.max() < 1e-6


def test_cls_parity_same_transfers(fid):
    T, _, delta, icl = fid
    g = T.cls_gpu(delta)
    assert np.max(np.abs(g[:, :2] / icl[:, :2] - 1)) < 1e-12
    assert np.max(np.abs(g[:, 2] - icl[:, 2]) / np.sqrt(icl[:, 0] * icl[:, 1])) < 1e-12


def test_end_to_end_cls(fid):
    T, _, _, icl = fid
    cls = np.zeros((1001, 4))
    p = fiducial(1000)
    import ctypes as C
    _lib.check(_lib.load().cambgpu_get_results(C.byref(p), 1000, _lib.dptr(cls)))
    ls = T.ls
    got = cls[ls]
    assert np.max(np.abs(got[:, 0] / icl[:, 0] - 1)) < 1e-5
    assert np.max(np.abs(got[:, 1] / icl[:, 1] - 1)) < 1e-5
    assert np.max(np.abs(got[:, 3] - icl[:, 2]) / np.sqrt(icl[:, 0] * icl[:, 1])) < 1e-5


def test_lensing_potential_source_parity():
    T = _lib.Tables(fiducial(400, lensing=True))
    src = orc.evolve_sources(T)
    g = T.evolve_sources_gpu()
    assert rel_peak(g, src, axis=0) < 1e-6
    delta = orc.los(T, src)
    gd = T.los_gpu(src)
    peak = np.max(np.abs(delta), axis=1, keepdims=True)
    m = np.abs(delta) > 1e-3 * peak
    assert (np.abs(gd - delta)[m] / np.abs(delta)[m]).max() < 1e-6
    icl = orc.cls(T, delta)
    gi = T.cls_gpu(delta)
    assert np.max(np.abs(gi[:, 3] / icl[:, 3] - 1)) < 1e-12


def test_batch_of_ragged_cosmologies_matches_oracle():
    """Seeded +-5% draws: every cosmology has its own k, tau and q grids."""
    ps = draws(4, seed=7, lmax=600)
    import ctypes as C
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    cls = np.zeros((len(ps), 601, 4))
    st = np.zeros(len(ps), dtype=np.int32)
    _lib.check(_lib.load().cambgpu_get_results_batch(arr, len(ps), 600, _lib.dptr(cls), _lib.iptr(st)))
    assert not st.any()
    sizes = set()
    for i, p in enumerate(ps):
        T = _lib.Tables(p)
        sizes.add((T.view.nk, T.view.ntau, T.view.nq))
        icl = orc.cls(T, orc.los(T, orc.evolve_sources(T)))
        got = cls[i][T.ls]
        assert np.max(np.abs(got[:, 0] / icl[:, 0] - 1)) < 1e-5
        assert np.max(np.abs(got[:, 1] / icl[:, 1] - 1)) < 1e-5
    assert len(sizes) > 1


@pytest.mark.parametrize("team", [32, 16, 8, 6, 1, 2, 3, 4, 5, 7])
def test_team_sizes_agree(fid, team):
    T, src, _, _ = fid
    lib = _lib.load()
    _lib.check(lib.cambgpu_set_ode_team(team))
    try:
        g = T.evolve_sources_gpu()
    finally:
        lib.cambgpu_set_ode_team(0)
    assert rel_peak(g, src, axis=0) < 1e-6


def test_invalid_batch_reports_error_without_fault():
    import ctypes as C
    lib = _lib.load()
    p = fiducial(300)
    p.omk = 0.05
    cls = np.zeros((301, 4))
    st = np.zeros(1, dtype=np.int32)
    rc = lib.cambgpu_get_results_batch(C.byref(p), 1, 300, _lib.dptr(cls), _lib.iptr(st))
    assert rc == 2 and st[0] == 2
    rc = lib.cambgpu_get_results_batch(C.byref(p), 0, 300, _lib.dptr(cls), _lib.iptr(st))
    assert rc == 2
    # the context is still usable afterwards
    test = fiducial(300)
    _lib.check(lib.cambgpu_get_results(C.byref(test), 300, _lib.dptr(cls)))
    assert np.all(np.isfinite(cls)) and cls[100, 0] > 0


def test_resident_batch_graph_replay_is_identical():
    """Repeated runs of a resident batch replay the stage sequence as a CUDA graph (captured
    on the second run); the C_l of the eager first run, the capturing run and a replay
    are identical, and a replay counts the graph's kernel launches."""
    ps = draws(3, seed=21, lmax=600, mnu_max=0.1)
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    lib = _lib.load()
    _lib.check(lib.cambgpu_batch_prepare(arr, len(ps)))
    try:
        outs = []
        for _ in range(3):
            lib.cambgpu_kernel_launches(1)
            _lib.check(lib.cambgpu_batch_run(None))
            launches = lib.cambgpu_kernel_launches(1)
            cls = np.zeros((len(ps), 601, 4))
            _lib.check(lib.cambgpu_batch_fetch(600, _lib.dptr(cls)))
            outs.append((cls, launches))
    finally:
        lib.cambgpu_batch_release()
    assert outs[0][1] > 0 and outs[1][1] == outs[0][1] and outs[2][1] == outs[0][1]
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][0], outs[2][0])


def test_results_stream_matches_blocking_calls():
    """get_results_stream (next batch's host tables built while the device runs this one)
    gives the same spectra as one blocking call per batch, and releases a prepared batch
    when the consumer stops early."""
    from camb_gb300 import model, results
    batches = [[model.set_params(lmax=500, DoLensing=False, mnu=0.0, H0=h, ombh2=0.022 + 0.0002 * i)
                for i in range(2)] for h in (66.0, 67.5, 69.0)]
    streamed = list(results.get_results_stream(batches))
    assert len(streamed) == 3
    for got, ps in zip(streamed, batches):
        want = results.get_results_batch(ps)
        for g, w in zip(got, want):
            assert np.array_equal(g.get_unlensed_scalar_cls(500), w.get_unlensed_scalar_cls(500))
    it = results.get_results_stream(batches)
    next(it)
    it.close()  # the second batch was being prepared: it is freed, nothing leaks or faults


def test_queue_orders_and_caps_give_identical_results():
    """Every k-mode is integrated independently, so the work-queue order (including the
    measured-cost order built from the previous run), the resident-block cap and the
    schedule (queue counter or static stride) change only which thread runs which mode,
    never a bit of the spectra of one kernel variant."""
    ps = draws(3, seed=5, lmax=500, mnu_max=0.1)
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    lib = _lib.load()
    _lib.check(lib.cambgpu_batch_prepare(arr, len(ps)))
    outs = {}
    try:
        for team, order, cap, sched in [(1, 0, 0, 0), (1, 2, 2, 0), (1, 3, 2, 0), (1, 3, 1, 0), (1, 1, 0, 0),
                                        (1, 2, 2, 1), (1, 0, 0, 1), (7, 2, 0, 0), (7, 2, 0, 1), (7, 3, 0, 1),
                                        (6, 0, 0, 0), (6, 0, 0, 1), (7, 4, 0, 1), (1, 4, 0, 1), (1, 4, 3, 1),
                                        (7, 4, 0, 0)]:
            _lib.check(lib.cambgpu_set_ode_team(team))
            _lib.check(lib.cambgpu_set_ode_launch(order, cap))
            _lib.check(lib.cambgpu_set_ode_schedule(sched))
            _lib.check(lib.cambgpu_batch_run(None))
            cls = np.zeros((len(ps), 501, 4))
            _lib.check(lib.cambgpu_batch_fetch(500, _lib.dptr(cls)))
            outs.setdefault(team, []).append(cls)
    finally:
        lib.cambgpu_set_ode_team(0)
        lib.cambgpu_set_ode_launch(-1, 0)
        lib.cambgpu_set_ode_schedule(-1)
        lib.cambgpu_batch_release()
    for runs in outs.values():
        for o in runs[1:]:
            assert np.array_equal(o, runs[0])


def test_first_run_on_the_cost_prior_is_identical():
    """A fresh batch of a kind that has run before starts on a balanced queue built from the
    previous batch's evaluations per ln q (the cost prior); like any queue it changes only
    which thread runs which mode.  The first run of a fresh batch on the prior, its second
    run on its own measured costs, and a run on the q-band order give the same spectra."""
    lib = _lib.load()
    first = draws(3, seed=5, lmax=500, mnu_max=0.1)
    second = draws(3, seed=6, lmax=500, mnu_max=0.1)
    outs = []
    try:
        _lib.check(lib.cambgpu_set_ode_team(7))
        _lib.check(lib.cambgpu_set_ode_schedule(1))
        for ps, order, runs in [(first, 4, 1), (second, 4, 2), (second, 2, 1)]:
            arr = (_lib.CambGpuParams * len(ps))(*ps)
            _lib.check(lib.cambgpu_set_ode_launch(order, 0))
            _lib.check(lib.cambgpu_batch_prepare(arr, len(ps)))
            for _ in range(runs):
                _lib.check(lib.cambgpu_batch_run(None))
                cls = np.zeros((len(ps), 501, 4))
                _lib.check(lib.cambgpu_batch_fetch(500, _lib.dptr(cls)))
                outs.append(cls)
            lib.cambgpu_batch_release()
    finally:
        lib.cambgpu_set_ode_team(0)
        lib.cambgpu_set_ode_launch(-1, 0)
        lib.cambgpu_set_ode_schedule(-1)
        lib.cambgpu_batch_release()
    assert np.array_equal(outs[1], outs[2]) and np.array_equal(outs[1], outs[3])
    assert not np.array_equal(outs[0], outs[1])  # different draws


def test_resident_batch_refuses_after_a_later_staging():
    """A one-shot call reuses the device arena: the resident batch then reports an error
    instead of computing on overwritten tables, and the library stays usable."""
    ps = draws(2, seed=9, lmax=400)
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    lib = _lib.load()
    _lib.check(lib.cambgpu_batch_prepare(arr, len(ps)))
    try:
        _lib.check(lib.cambgpu_batch_run(None))
        cls = np.zeros((401, 4))
        one = fiducial(400)
        _lib.check(lib.cambgpu_get_results(C.byref(one), 400, _lib.dptr(cls)))
        assert lib.cambgpu_batch_run(None) == 2
        out = np.zeros((len(ps), 401, 4))
        assert lib.cambgpu_batch_fetch(400, _lib.dptr(out)) == 2
    finally:
        lib.cambgpu_batch_release()
    _lib.check(lib.cambgpu_batch_prepare(arr, len(ps)))
    _lib.check(lib.cambgpu_batch_run(None))
    lib.cambgpu_batch_release()


def test_wide_parameter_box_against_the_oracle():
    """Twelve cosmologies far outside the benchmark's +-5% box (H0 55-80, ombh2 0.018-0.026,
    omch2 0.09-0.15, tau 0.03-0.12, ns 0.90-1.02, nrun -0.02-0.02, N_eff 2.5-4, one massive
    eigenstate of 0-0.5 eV or three degenerate ones), lmax 800, as one batch through
    cambgpu_get_results_batch (FP64): C_l at the sampled l within 1e-5 of the oracle's, so
    the switch logic, the hierarchy sizes and the massive-neutrino momentum bins hold
    outside the draws the other tests use."""
    rng = np.random.default_rng(77)
    ps = []
    for i in range(12):
        p = fiducial(800)
        p.H0 = rng.uniform(55, 80)
        p.ombh2 = rng.uniform(0.018, 0.026)
        p.omch2 = rng.uniform(0.09, 0.15)
        p.optical_depth = rng.uniform(0.03, 0.12)
        p.ns = rng.uniform(0.90, 1.02)
        p.nrun = rng.uniform(-0.02, 0.02)
        p.nnu = rng.uniform(2.5, 4.0)
        if i % 3:
            p.mnu = rng.uniform(0.0, 0.5)
            p.num_massive_neutrinos = 3 if i % 3 == 2 else 1
        ps.append(p)
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    lib = _lib.load()
    old = lib.cambgpu_get_precision()
    _lib.check(lib.cambgpu_set_precision(0))
    try:
        cls = np.zeros((len(ps), 801, 4))
        st = np.zeros(len(ps), dtype=np.int32)
        _lib.check(lib.cambgpu_get_results_batch(arr, len(ps), 800, _lib.dptr(cls), _lib.iptr(st)))
    finally:
        lib.cambgpu_set_precision(old)
    assert np.all(st == 0)
    for i, p in enumerate(ps):
        T = _lib.Tables(p)
        icl = orc.cls(T, orc.los(T, orc.evolve_sources(T)))
        got = cls[i][T.ls]
        assert np.max(np.abs(got[:, 0] / icl[:, 0] - 1)) < 1e-5, i
        assert np.max(np.abs(got[:, 1] / icl[:, 1] - 1)) < 1e-5, i
        assert np.max(np.abs(got[:, 3] - icl[:, 2]) / np.sqrt(icl[:, 0] * icl[:, 1])) < 1e-5, i


def test_concurrent_host_threads_get_the_sequential_results():
    """Four host threads calling cambgpu_get_spectra_batch at once (each its own batch, two
    calls each): the host tables build in parallel, the device work serialises on the
    library's lock, and every thread gets exactly the spectra of a sequential call."""
    from concurrent.futures import ThreadPoolExecutor
    lib = _lib.load()
    batches = [draws(2, seed=400 + i, lmax=600, mnu_max=0.1 * (i % 2)) for i in range(4)]

    def run(ps):
        arr = (_lib.CambGpuParams * len(ps))(*ps)
        cls = np.zeros((len(ps), 601, 4))
        st = np.zeros(len(ps), dtype=np.int32)
        _lib.check(lib.cambgpu_get_spectra_batch(arr, len(ps), 600, _lib.dptr(cls), None, None, None, _lib.iptr(st)))
        return cls

    want = [run(ps) for ps in batches]
    with ThreadPoolExecutor(4) as ex:
        got = list(ex.map(run, batches + batches))
    for i, g in enumerate(got):
        assert np.array_equal(g, want[i % 4]), i
