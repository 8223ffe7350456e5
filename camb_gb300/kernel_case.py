"""Fixed device workloads for profiler captures of single kernels.

    python -m camb_gb300.kernel_case <case>

stages one batch on the device once and runs the whole device pipeline (ODE, source
spline, line-of-sight projection, C_l) four times, printing the stage times of the
last run.  Under ncu, `-k regex:<kernel> -s 3 -c 1` then captures the fourth launch of
that kernel, after three warm launches.  Cases:

  warp1        one massless cosmology, lmax 1000, warp per mode (team 6)
  lens1        one cosmology with mnu 0.06 eV, lensed to lmax 2500 (+200), default kernel
  thread8      8 draws of the lmax-2500 workload, thread per mode (team 2)
  thread32     32 draws, thread per mode compiled for 2 blocks/SM (team 7), queue
               order 2 (q bands), static-stride schedule: the headline ODE
               configuration on a case small enough for multi-pass counter captures
  thread96/128 96 / 128 draws, team 1, queue order 2, 2 resident blocks/SM
  thread256    the 256 draws, team 1, queue order 2, 2 resident blocks/SM
  thread256r   the 256 draws, team 7, queue order 2, queue-counter schedule
  thread256s   the 256 draws, team 7, queue order 2, static-stride schedule (the
               configuration the benchmark's autotuner picks)
  team<T>_<N>[_o<order>][_s<schedule>][_c<cap>]
               N draws on ODE team code T, optionally with a queue order, a schedule
               and a resident-block cap (e.g. team7_256_o2_s1); unset parts keep the
               tuned defaults
  tc<N>        N lensed draws (lmax 2500 + 200) on grids shared by the batch, tensor-core
               projection (precision 2); fc<N> the same with the FP64 projection
  fp64pipe     the FP64 issue model (cambgpu_probe_fp64_pipe): lane FMAs per SM cycle for
               1-16 warps per SM, partially active warps and 1/4/8 independent chains
"""
import json
import sys

import numpy as np

from . import _lib
from .workload import batch_draws


def fp64_pipe():
    """Lane FMAs per SM cycle of the DFMA probe over warps per SM, active lanes, chains."""
    import ctypes as C
    lib = _lib.load()
    rows = []
    cases = [(w, 32, 8) for w in (1, 2, 3, 4, 6, 8, 16)] + [(1, l, 8) for l in (1, 8, 16)] + \
            [(4, l, 8) for l in (1, 8, 16)] + [(1, 32, c) for c in (1, 4)] + [(4, 32, c) for c in (1, 4)]
    for w, l, c in cases:
        v = C.c_double()
        _lib.check(lib.cambgpu_probe_fp64_pipe(w, l, c, C.byref(v)))
        rows.append({"warps_per_sm": w, "active_lanes": l, "chains": c, "lane_fma_per_sm_cycle": round(v.value, 4),
                     "cycles_per_warp_dfma": round(w * l / v.value, 1)})
    out = {"kernel_case": "fp64pipe", "rows": rows}
    print(json.dumps(out))
    return out


def run(name, runs=4):
    lib = _lib.load()
    sched = 0
    if name == "fp64pipe":
        return fp64_pipe()
    if name.startswith(("tc", "fc")):
        ps = batch_draws(int(name[2:]), 2500, seed=5000)
        for p in ps:
            p.do_lensing, p.max_l = 1, 2700
            p.max_eta_k = 2.5 * 2700
        arr = (_lib.CambGpuParams * len(ps))(*ps)
        _lib.check(lib.cambgpu_set_precision(2 if name.startswith("tc") else 0))
        _lib.check(lib.cambgpu_batch_prepare_shared(arr, len(ps), None))
        ms = np.zeros(3)
        for _ in range(runs):
            _lib.check(lib.cambgpu_batch_run(_lib.dptr(ms)))
        lib.cambgpu_batch_release()
        lib.cambgpu_set_precision(1)
        out = {"kernel_case": name, "ode_ms": ms[0], "spline_los_ms": ms[1], "cls_ms": ms[2]}
        print(json.dumps(out))
        return out
    if name == "lens1":  # one cosmology, mnu 0.06 eV, lensed to lmax 2500 (+200), the default kernel choice
        p = _lib.default_params()
        p.H0, p.ombh2, p.omch2, p.optical_depth, p.As, p.ns = 67.5, 0.022, 0.122, 0.06, 2.1e-9, 0.965
        p.nnu, p.mnu, p.num_massive_neutrinos = 3.046, 0.06, 1
        p.do_lensing, p.max_l, p.max_eta_k = 1, 2700, 2.5 * 2700
        ps, team, order, cap = [p], 0, -1, 0
    elif name == "warp1":
        p = _lib.default_params()
        p.H0, p.ombh2, p.omch2, p.optical_depth, p.As, p.ns = 67.5, 0.022, 0.122, 0.06, 2.1e-9, 0.965
        p.nnu, p.mnu, p.num_massive_neutrinos = 3.046, 0.0, 1
        p.max_l, p.max_eta_k = 1000, 2500
        ps, team, order, cap = [p], 6, -1, 0
    elif name == "thread8":
        ps, team, order, cap = batch_draws(8, 2500, seed=7), 2, -1, 0
    elif name == "thread32":
        ps, team, order, cap, sched = batch_draws(32, 2500, seed=1000), 7, 2, 0, 1
    elif name in ("thread96", "thread128"):
        ps, team, order, cap = batch_draws(int(name[6:]), 2500, seed=1000), 1, 2, 2
    elif name == "thread256r":
        ps, team, order, cap = batch_draws(256, 2500, seed=1000), 7, 2, 0
    elif name == "thread256s":
        ps, team, order, cap, sched = batch_draws(256, 2500, seed=1000), 7, 2, 0, 1
    elif name == "thread256":
        ps, team, order, cap = batch_draws(256, 2500, seed=1000), 1, 2, 2
    elif name.startswith("team"):
        parts = name[4:].split("_")
        order, sched, cap = -1, -1, 0
        for extra in parts[2:]:
            if extra[0] == "o":
                order = int(extra[1:])
            elif extra[0] == "s":
                sched = int(extra[1:])
            elif extra[0] == "c":
                cap = int(extra[1:])
        ps, team = batch_draws(int(parts[1]), 2500, seed=1000), int(parts[0])
    else:
        raise SystemExit(f"unknown case {name}")
    arr = (_lib.CambGpuParams * len(ps))(*ps)
    _lib.check(lib.cambgpu_set_ode_team(team))
    _lib.check(lib.cambgpu_set_ode_launch(order, cap))
    _lib.check(lib.cambgpu_set_ode_schedule(sched))
    _lib.check(lib.cambgpu_set_precision(1))
    _lib.check(lib.cambgpu_batch_prepare(arr, len(ps)))
    ms = np.zeros(3)
    for _ in range(runs):
        _lib.check(lib.cambgpu_batch_run(_lib.dptr(ms)))
    evals = lib.cambgpu_last_ode_evals()
    lib.cambgpu_batch_release()
    out = {"kernel_case": name, "ode_ms": ms[0], "spline_los_ms": ms[1], "cls_ms": ms[2], "ode_evals": int(evals)}
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    run(sys.argv[1] if len(sys.argv) > 1 else "thread32")
