"""The split hi/lo BF16 tensor-core projection (precision 2) of batches on shared grids,
against the FP64 projection on the same grids, through the C ABI: unlensed TT, EE, TE to
lmax 1000 and lensed TT, EE, BB, TE with the lensing potential to lmax 2500 (+200 margin),
relative error within 1e-4 at every l (TE against sqrt(TT EE)).  The FP64 projection of
the shared-grid batch itself matches the oracle run on the same shared-grid tables."""
import ctypes as C

import numpy as np
import pytest

from camb_gb300 import _lib
from camb_gb300.workload import batch_draws
from oracle import oracle as orc
from tests.test_cpu_shared_grid import shared_tables

pytestmark = pytest.mark.gpu


def run_shared(ps, precisions, lmax_out, lensed=False):
    lib = _lib.load()
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    nchi = C.c_int()
    _lib.check(lib.cambgpu_batch_prepare_shared(arr, len(ps), C.byref(nchi)))
    old = lib.cambgpu_get_precision()
    out = {}
    try:
        for prec in precisions:
            _lib.check(lib.cambgpu_set_precision(prec))
            _lib.check(lib.cambgpu_batch_run(None))
            n = len(ps)
            unl = np.zeros((n, lmax_out + 1, 4))
            if lensed:
                len_ = np.zeros((n, lmax_out + 1, 4))
                pot = np.zeros((n, lmax_out + 1, 3))
                lml = np.zeros(n, dtype=np.int32)
                _lib.check(lib.cambgpu_batch_spectra_from_transfer(None, None, None, None, lmax_out, _lib.dptr(unl),
                                                                   _lib.dptr(len_), _lib.dptr(pot), _lib.iptr(lml)))
                out[prec] = (unl, len_, pot, lml)
            else:
                _lib.check(lib.cambgpu_batch_fetch(lmax_out, _lib.dptr(unl)))
                out[prec] = (unl,)
    finally:
        lib.cambgpu_set_precision(old)
        lib.cambgpu_batch_release()
    return out, nchi.value


def rel(a, b):
    return np.max(np.abs(a / b - 1))


def test_unlensed_tensor_projection_matches_fp64_on_shared_grids():
    ps = batch_draws(4, 1000, seed=21)
    out, nchi = run_shared(ps, (0, 2), 1000)
    ref, got = out[0][0][:, 2:], out[2][0][:, 2:]
    assert nchi > 100
    assert rel(got[..., 0], ref[..., 0]) < 1e-4
    assert rel(got[..., 1], ref[..., 1]) < 1e-4
    assert np.max(np.abs(got[..., 3] - ref[..., 3]) / np.sqrt(ref[..., 0] * ref[..., 1])) < 1e-4
    # the FP64 projection of the shared-grid batch against the oracle on the same tables
    ts, _ = shared_tables(ps)
    T = ts[1]
    icl = orc.cls(T, orc.los(T, orc.evolve_sources(T)))
    g = out[0][0][1][T.ls]
    assert rel(g[:, 0], icl[:, 0]) < 1e-5 and rel(g[:, 1], icl[:, 1]) < 1e-5


def test_lensed_tensor_projection_matches_fp64_on_shared_grids():
    ps = batch_draws(3, 2500, seed=22)
    for p in ps:
        p.do_lensing = 1
        p.max_l = 2700
        p.max_eta_k = 2.5 * 2700
    out, _ = run_shared(ps, (0, 2), 2700, lensed=True)
    unl0, len0, pot0, lml0 = out[0]
    unl2, len2, pot2, lml2 = out[2]
    assert np.array_equal(lml0, lml2)
    for i in range(len(ps)):
        n = int(lml0[i])
        r, g = len0[i, 2:n + 1], len2[i, 2:n + 1]
        assert rel(g[:, 0], r[:, 0]) < 1e-4
        assert rel(g[:, 1], r[:, 1]) < 1e-4
        assert rel(g[:, 2], r[:, 2]) < 1e-4
        assert np.max(np.abs(g[:, 3] - r[:, 3]) / np.sqrt(r[:, 0] * r[:, 1])) < 1e-4
        assert rel(pot2[i, 2:2501, 0], pot0[i, 2:2501, 0]) < 1e-4


def test_tensor_projection_several_cosmology_tiles():
    """130 draws: two 128-cosmology tiles, the second nearly empty."""
    ps = batch_draws(130, 600, seed=23)
    out, _ = run_shared(ps, (0, 2), 600)
    ref, got = out[0][0][:, 2:], out[2][0][:, 2:]
    assert rel(got[..., 0], ref[..., 0]) < 1e-4
    assert rel(got[..., 1], ref[..., 1]) < 1e-4
    assert np.max(np.abs(got[..., 3] - ref[..., 3]) / np.sqrt(ref[..., 0] * ref[..., 1])) < 1e-4


def test_public_shared_grid_api_tensor_against_fp64_and_native_grids():
    """get_results_batch_shared (the Python surface) with the tensor projection: lensed TT,
    EE, BB within 1e-4 of the FP64 projection on the same shared grids, and within 3e-3
    of get_results_batch on each cosmology's own grids below l = 2000."""
    import camb_gb300 as cg
    ps = [cg.set_params(lmax=2000, H0=h, ombh2=b, omch2=c, mnu=m)
          for h, b, c, m in ((67.5, 0.0224, 0.120, 0.06), (70.0, 0.0220, 0.115, 0.12), (65.0, 0.0228, 0.125, 0.0))]
    before = _lib.load().cambgpu_get_precision()
    got = cg.get_results_batch_shared(ps, projection="tensor")
    ref = cg.get_results_batch_shared(ps, projection="fp64")
    nat = cg.get_results_batch(ps)
    for g, r, n in zip(got, ref, nat):
        gl, rl, nl = (x.get_lensed_scalar_cls(2000, raw_cl=True)[2:] for x in (g, r, n))
        for c in range(3):
            assert rel(gl[:, c], rl[:, c]) < 1e-4
            assert rel(rl[:, c], nl[:, c]) < 3e-3
        gp, rp = g.get_lens_potential_cls(2000, raw_cl=True)[2:], r.get_lens_potential_cls(2000, raw_cl=True)[2:]
        assert rel(gp[:, 0], rp[:, 0]) < 1e-4
    assert _lib.load().cambgpu_get_precision() == before  # the caller's precision is restored


def test_tensor_projection_with_two_l_tiles():
    """lSampleBoost 2 at lmax 2500 (+200, lensed) samples 155 l, more than one 128-row tile
    of the tensor-core product: the l tiles run side by side in the grid, and TT, EE, BB
    and phi-phi stay within 1e-4 of the FP64 projection on the same shared grids."""
    ps = batch_draws(3, 2500, seed=31)
    for p in ps:
        p.do_lensing, p.max_l, p.max_eta_k = 1, 2700, 2.5 * 2700
        p.lSampleBoost = 2.0
    out, _ = run_shared(ps, (0, 2), 2700, lensed=True)
    (_, ref_l, ref_p, lml), (_, got_l, got_p, _) = out[0], out[2]
    assert _lib.Tables(ps[0]).view.nl > 128
    L = int(lml.min())
    for c in range(3):
        assert rel(got_l[:, 2:L, c], ref_l[:, 2:L, c]) < 1e-4, c
    assert rel(got_p[:, 2:2501, 0], ref_p[:, 2:2501, 0]) < 1e-4
