"""Host-only entry points of the C ABI on CPU (no device call is made): building a batch's
host tables ahead of its device run, error codes and per-cosmology status for invalid
parameters, and the argument checks of the ODE controls."""
import ctypes
import ctypes as C

import numpy as np

from camb_gb300 import _lib
from tests.cosmologies import draws, fiducial


def test_prepare_tables_builds_and_frees(lib):
    ps = draws(3, seed=3, lmax=500, mnu_max=0.1)
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    h = C.c_void_p()
    st = np.full(len(ps), -1, dtype=np.int32)
    _lib.check(lib.cambgpu_prepare_tables(arr, len(ps), C.byref(h), _lib.iptr(st)))
    assert h.value and not st.any()
    lib.cambgpu_free_prepared(h)


def test_prepare_tables_reports_bad_members(lib):
    bad = fiducial(500)
    bad.omk = 0.05  # curved: not part of the flat path
    ps = [fiducial(500), bad]
    arr = (_lib.CambGpuParams * 2)(*ps)
    h = C.c_void_p()
    st = np.zeros(2, dtype=np.int32)
    rc = lib.cambgpu_prepare_tables(arr, 2, C.byref(h), _lib.iptr(st))
    assert rc == 2 and not h.value
    assert st[0] == 0 and st[1] == 2
    assert lib.cambgpu_last_error()
    assert lib.cambgpu_prepare_tables(arr, 0, C.byref(h), None) == 2
    # the device half refuses a missing batch before touching the device
    assert lib.cambgpu_get_spectra_prepared(None, 500, None, None, None, None, None) == 2


def test_ode_controls_validate_arguments(lib):
    assert lib.cambgpu_set_ode_team(9) == 2
    assert lib.cambgpu_set_ode_team(-1) == 2
    assert lib.cambgpu_set_ode_launch(5, 0) == 2
    assert lib.cambgpu_set_ode_launch(4, 0) == 0
    assert lib.cambgpu_set_ode_launch(2, -1) == 2
    for team in (0, 1, 5, 6, 7, 8, 16, 32):
        assert lib.cambgpu_set_ode_team(team) == 0
    assert lib.cambgpu_set_ode_launch(3, 2) == 0
    assert lib.cambgpu_set_ode_team(0) == 0 and lib.cambgpu_set_ode_launch(-1, 0) == 0
    assert lib.cambgpu_set_ode_schedule(2) == 2 and lib.cambgpu_set_ode_schedule(-2) == 2
    for sched in (0, 1, -1):
        assert lib.cambgpu_set_ode_schedule(sched) == 0


def test_fp64_pipe_probe_validates_arguments(lib):
    import ctypes
    v = ctypes.c_double()
    assert lib.cambgpu_probe_fp64_pipe(0, 32, 8, ctypes.byref(v)) == 2
    assert lib.cambgpu_probe_fp64_pipe(4, 33, 8, ctypes.byref(v)) == 2
    assert lib.cambgpu_probe_fp64_pipe(4, 32, 3, ctypes.byref(v)) == 2
    assert lib.cambgpu_probe_fp64_pipe(4, 32, 8, None) == 2


def test_gemm_bf16x3_validates_arguments(lib):
    fp = ctypes.POINTER(ctypes.c_float)
    a = np.zeros(4, dtype=np.float32)
    p = a.ctypes.data_as(fp)
    assert lib.cambgpu_gemm_bf16x3(p, p, 0, 1, 1, p) == 2
    assert lib.cambgpu_gemm_bf16x3(p, p, 1, 1, 70000, p) == 2
    assert lib.cambgpu_gemm_bf16x3(None, p, 1, 1, 1, p) == 2


def test_noalloc_rejects_oversized_problem_before_any_device_call(lib):
    """The allocation-free LOS entry point checks the problem against its fixed scratch
    array first: an oversized problem is refused with code 2 and a message naming the
    sizes, without touching the device (so this runs without a GPU).  No buffer is read:
    the pointers only have to be non-null."""
    T = _lib.Tables(draws(1, seed=5, lmax=300)[0])
    dv = _lib.CambGpuTables.from_buffer_copy(T.view)
    dv.nk = 1 << 20
    buf = np.zeros(8)
    rc = lib.cambgpu_los_flat_noalloc(C.byref(dv), _lib.dptr(buf), _lib.dptr(buf), None)
    assert rc == 2
    msg = lib.cambgpu_last_error().decode()
    assert "scratch" in msg and str(1 << 20) in msg
    assert lib.cambgpu_los_flat_noalloc(None, _lib.dptr(buf), _lib.dptr(buf), None) == 2


def test_noalloc_rejects_long_time_grid_before_any_device_call(lib):
    """A time grid whose shared-memory staging (ntau*44 + 64 bytes) exceeds the projection
    kernel's 160 KiB is refused with code 2 and a message naming ntau, before any device
    call (so this runs without a GPU)."""
    T = _lib.Tables(draws(1, seed=5, lmax=300)[0])
    dv = _lib.CambGpuTables.from_buffer_copy(T.view)
    dv.ntau = 4000
    buf = np.zeros(8)
    rc = lib.cambgpu_los_flat_noalloc(C.byref(dv), _lib.dptr(buf), _lib.dptr(buf), None)
    assert rc == 2
    msg = lib.cambgpu_last_error().decode()
    assert "ntau=4000" in msg and "shared memory" in msg


def test_results_with_transfers_validates_before_any_device_call(lib):
    """cambgpu_get_results_with_transfers wants the CMB and transfer functions in every member
    and one redshift count across the batch; anything else is code 2 with a message,
    before any device call."""
    p = fiducial(300)
    p.want_transfer, p.num_transfer_redshifts = 1, 1
    p.transfer_redshifts[0] = 0.0
    q = fiducial(300)  # CMB only
    for ps in ([p, q], [q]):
        arr = (_lib.CambGpuParams * len(ps))(*ps)
        st = np.zeros(len(ps), dtype=np.int32)
        rc = lib.cambgpu_get_results_with_transfers(arr, len(ps), 300, None, None, None, None, 16, None, None, None,
                                                    None, _lib.iptr(st))
        assert rc == 2 and b"want_cls = want_transfer = 1" in lib.cambgpu_last_error()
    r = fiducial(300)
    r.want_transfer, r.num_transfer_redshifts = 1, 2
    r.transfer_redshifts[0], r.transfer_redshifts[1] = 1.0, 0.0
    arr = (_lib.CambGpuParams * 2)(p, r)
    rc = lib.cambgpu_get_results_with_transfers(arr, 2, 300, None, None, None, None, 16, None, None, None, None, None)
    assert rc == 2 and b"same redshift count" in lib.cambgpu_last_error()
