"""The allocation-free LOS entry point, for callers that cannot allocate device memory
(code inside a framework that owns all device memory, or a service that must not
allocate after start-up).  The caller -- here the test, through torch -- owns every
input and output buffer on the device; the library's only scratch is its static
device array.  The output must match the regular entry point cambgpu_los_flat
(host buffers) within the parity tolerance, on two calls in a row with different
cosmologies (so stale scratch from the first call would show up in the second).

Kept in a file that pytest collects last so that a stop-at-first-failure run has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from camb_gb300 import _lib
from tests.cosmologies import draws

pytestmark = pytest.mark.gpu


def _device_view(T, torch):
    """A copy of T.view whose array pointers refer to device copies (kept alive in `keep`)."""
    v = T.view
    dv = _lib.CambGpuTables.from_buffer_copy(v)
    keep = []

    def up(name, n, dtype=np.float64):
        a = np.ctypeslib.as_array(getattr(v, name), shape=(n,)).astype(dtype, copy=True)
        t = torch.from_numpy(a).cuda()
        keep.append(t)
        return t.data_ptr()

    dv.q_evolve = C.cast(C.c_void_p(up("q_evolve", v.nk)), C.POINTER(C.c_double))
    dv.tau_points = C.cast(C.c_void_p(up("tau_points", v.ntau)), C.POINTER(C.c_double))
    dv.tau_dpoints = C.cast(C.c_void_p(up("tau_dpoints", v.ntau)), C.POINTER(C.c_double))
    dv.q_int = C.cast(C.c_void_p(up("q_int", v.nq)), C.POINTER(C.c_double))
    dv.ls = C.cast(C.c_void_p(up("ls", v.nl, np.int32)), C.POINTER(C.c_int))
    dv.bess_x = C.cast(C.c_void_p(up("bess_x", v.num_xx)), C.POINTER(C.c_double))
    dv.bessel_horner = C.cast(C.c_void_p(up("bessel_horner", v.nl * (v.num_xx - 1) * 4)), C.POINTER(C.c_double))
    return dv, keep


def test_los_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = _lib.load()
    for p in draws(2, seed=99, lmax=700):
        T = _lib.Tables(p)
        v = T.view
        src = T.evolve_sources_gpu()
        ref = T.los_gpu(src)  # existing entry point, host buffers
        dv, keep = _device_view(T, torch)
        d_src = torch.from_numpy(np.ascontiguousarray(src)).cuda()
        d_out = torch.full((v.nq, v.nl, v.nsrc), float("nan"), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.cambgpu_los_flat_noalloc(C.byref(dv), C.c_void_p(d_src.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                          C.c_void_p(stream))
        assert rc == 0, lib.cambgpu_last_error()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        peak = np.max(np.abs(ref), axis=1, keepdims=True)
        m = np.abs(ref) > 1e-3 * peak
        assert np.all(np.isfinite(got))
        assert (np.abs(got - ref)[m] / np.abs(ref)[m]).max() < 1e-6
        assert np.max(np.abs(got[~m] - ref[~m])) <= 1e-3 * peak.max()
        del keep


def test_los_noalloc_rejects_oversized_problem():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = _lib.load()
    T = _lib.Tables(draws(1, seed=5, lmax=300)[0])
    dv, keep = _device_view(T, torch)
    dv.nk = 1 << 20  # 5*nk + ntau*nsrc*nk far beyond the 16 MiB scratch; nothing is launched
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.cambgpu_los_flat_noalloc(C.byref(dv), C.c_void_p(d.data_ptr()), C.c_void_p(d.data_ptr()), None)
    assert rc == 2


def test_los_noalloc_rejects_host_buffers():
    """Every buffer must be device memory: a host array passed as the sources is refused
    with code 2 before anything is launched, and the context stays usable."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    lib = _lib.load()
    T = _lib.Tables(draws(1, seed=5, lmax=300)[0])
    dv, keep = _device_view(T, torch)
    host_src = np.zeros((T.view.ntau, T.view.nsrc, T.view.nk))
    d_out = torch.zeros((T.view.nq, T.view.nl, T.view.nsrc), dtype=torch.float64, device="cuda")
    rc = lib.cambgpu_los_flat_noalloc(C.byref(dv), _lib.dptr(host_src), C.c_void_p(d_out.data_ptr()), None)
    assert rc == 2
    assert "linear_src_dev" in lib.cambgpu_last_error().decode()
    dv.bess_x = T.view.bess_x  # a host table inside the view
    d_src = torch.zeros(host_src.shape, dtype=torch.float64, device="cuda")
    rc = lib.cambgpu_los_flat_noalloc(C.byref(dv), C.c_void_p(d_src.data_ptr()), C.c_void_p(d_out.data_ptr()), None)
    assert rc == 2
    assert "bess_x" in lib.cambgpu_last_error().decode()
    torch.cuda.synchronize()
    del keep
