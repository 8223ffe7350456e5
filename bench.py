"""Benchmark: cosmologies/s of the GB300 scalar-perturbation path at <=1e-4 relative C_l
error.

One step = one batch of B seeded cosmology draws (each of ombh2, omch2, H0, tau,
As, ns uniform in fiducial +-5%, one massive neutrino eigenstate with mnu uniform in
0-0.2 eV, unlensed scalar C_l to lmax=2500) through the hot path: per-k ODE sources, source k-spline + flat
line-of-sight projection, C_l.  `value` times the device pipeline on tables already
resident in HBM (CUDA events on the library's stream); `e2e` times the C ABI calls a
user makes for a stream of batches (host parameters in, host C_l out, host table
build and host<->device copies inside the timed region; the next batch's host tables
are built while the device runs the current one), with the single blocking call
cambgpu_get_results_batch reported beside it.  The batch is timed twice on the
device: the FP64 form (reported as fp64_form) and the timed form (--precision, default 1:
FP32 line-of-sight projection), whose C_l error against the FP64 form over the whole
batch and against the FP64 CPU restatement is reported beside the number.

--impl reference times the reference's CPU path for the same workload on this
machine's host cores: the C++ restatement of the reference (oracle/) on every core, in
two forms -- OpenMP over k-modes for one cosmology at a time, as the reference
parallelises it (cmbmain.f90:205-209, 287-291), and one cosmology per thread -- and
reports the faster.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lmax", type=int, default=2500)
    ap.add_argument("--team", type=int, default=0)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=4)
    ap.add_argument("--mnu-max", type=float, default=0.2)
    ap.add_argument("--precision", type=int, default=1, choices=[0, 1],
                    help="timed form: 0 FP64 throughout, 1 mixed-precision line-of-sight projection")
    ap.add_argument("--lensed-batch", type=int, default=0,
                    help="instead of the headline run: N lensed draws (lmax 2500 + 200 margin) on grids shared by "
                         "the batch through the FP64, mixed FP32 and tensor-core BF16x3 projections, device time "
                         "per form and C_l errors per l band (and the shift from each draw's own grids)")
    return ap.parse_args()


# the benchmark's metric: `value` is the batched cosmologies/s (unlensed scalar TT/EE/TE);
# the line also carries the plain GPU form ("batched_vs_plain_gpu") and grads/s ("gradients")
METRIC = "cosmologies/s to l=2500 at <=1e-4 rel C_l err, batched vs plain GPU; grads/s"


def plain_form_rate(n=3, lmax=2500, seed=1000, mnu_max=0.2):
    """The plain GPU form: one cosmology per blocking call, FP64 throughout (no mixed
    precision), draws of the same workload, host tables and copies included."""
    from camb_gb300 import _lib
    lib = _lib.load()
    ps = workload(n + 1, lmax, seed=seed, mnu_max=mnu_max)
    old = lib.cambgpu_get_precision()
    _lib.check(lib.cambgpu_set_precision(0))
    cls = np.zeros((lmax + 1, 4))
    try:
        _lib.check(lib.cambgpu_get_results(C.byref(ps[0]), lmax, _lib.dptr(cls)))
        t0 = time.perf_counter()
        for p in ps[1:]:
            _lib.check(lib.cambgpu_get_results(C.byref(p), lmax, _lib.dptr(cls)))
        t = time.perf_counter() - t0
    finally:
        lib.cambgpu_set_precision(old)
    return n / t


# DRAM bytes (read + write) of one ODE launch of the headline workload per (team code, queue
# order): ncu dram__bytes_read.sum + dram__bytes_write.sum of the fourth ODE launch of
# `python -m camb_gb300.kernel_case team7_256_o<order>_s1` (static stride), one pass each
# (profiles/ode_thread_kernel_dram_batch256_lmax2500.md)
ODE_TRAFFIC = {
    (7, 4): (911.95e9 + 442.84e9, "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 256-draw ODE launch "
                                  "(team 7, balanced queue order 4, static stride; kernel case team7_256_o4_s1)"),
}
# FP64 flops per right-hand-side evaluation (2 DFMA + DMUL + DADD thread instructions,
# stage combinations, error norm and source output included), ncu on the 32-draw case of
# this workload (kernel case thread32, profiles/ode_thread_kernel_batch32_lmax2500.md)
FLOPS_PER_EVAL = 1165
NOMINAL_FP64_TFLOPS = 152 * 2.07e9 * 4 / 1e12  # SMs x max SM clock x 4 flop per cycle


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def stream_steps(lib, arr, n, steps, lmax, cls, st, first=None):
    """steps batches through the C ABI in the stream's steady state: while batch k is
    staged, run and read back, a host thread builds the host tables of batch k+1 (and
    releases those of batch k).  `first`: the first batch's tables, built before the
    caller's timer (the pipeline fill); the loop then builds one batch ahead of the last,
    so each timed step still pays for one batch's host tables."""
    from concurrent.futures import ThreadPoolExecutor
    from camb_gb300 import _lib

    def prepare():
        h = C.c_void_p()
        ps = np.zeros(n, dtype=np.int32)
        _lib.check(lib.cambgpu_prepare_tables(arr, n, C.byref(h), _lib.iptr(ps)))
        return h

    with ThreadPoolExecutor(1) as ex:
        fut = ex.submit(prepare) if first is None else None
        nxt = first
        for k in range(steps):
            h = fut.result() if nxt is None else nxt
            nxt = None
            if first is not None or k + 1 < steps:
                fut = ex.submit(prepare)
            try:
                _lib.check(lib.cambgpu_get_spectra_prepared(h, lmax, _lib.dptr(cls), None, None, None, _lib.iptr(st)))
            finally:
                ex.submit(lib.cambgpu_free_prepared, h)  # released on the host thread too
        if first is not None:  # the batch built ahead of the last step
            ex.submit(lib.cambgpu_free_prepared, fut.result())


def prepare_first(lib, arr, n):
    """The first batch's host tables of a stream (before the timer: the pipeline fill)."""
    from camb_gb300 import _lib
    h = C.c_void_p()
    ps = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_prepare_tables(arr, n, C.byref(h), _lib.iptr(ps)))
    return h


def gradient_rate(n=64, lmax=2500, seed=3000, mnu_max=0.2):
    """Gradients dC_l/d(ombh2, omch2, H0, tau, As, ns) of n seeded draws through
    camb_gb300.gradients (central differences: 9 cosmologies per gradient in one batch),
    one warm-up call and one timed call, wall clock including the host tables."""
    from camb_gb300 import gradients, model
    rng = np.random.default_rng(seed)
    ps = []
    for _ in range(n):
        f = lambda v: v * (1 + 0.05 * (2 * rng.random() - 1))  # noqa: E731
        ps.append(model.set_params(lmax=lmax, DoLensing=False, H0=f(67.5), ombh2=f(0.022), omch2=f(0.122),
                                   tau=f(0.06), As=f(2.1e-9), ns=f(0.965), mnu=mnu_max * rng.random(),
                                   nnu=3.046))
    gradients.cl_gradients(ps[:4])
    t0 = time.perf_counter()
    cls, g = gradients.cl_gradients(ps)
    t = time.perf_counter() - t0
    out = {"value": n / t, "unit": "gradients/s (dC_l/d 6 parameters, l <= %d, unlensed)" % lmax, "batch": n,
           "seconds": t, "method": "central differences through the batched pipeline: ombh2, omch2, H0, tau "
                                   "re-evolved (+-1e-4 relative, 9 cosmologies per gradient in one launch, FP64 "
                                   "projection); As, ns by reweighting the resident transfer functions"}
    out.update(gradient_checks(ps[:2], g[:2]))
    out["cpu"] = cpu_gradient_rate(ps[:4])
    return out


def cpu_gradient_rate(ps):
    """The same central differences on the host cores: each gradient's 9 members (the
    draw and +-1e-4 in ombh2, omch2, H0, tau) through the CPU restatement, one cosmology
    per thread, host tables included (As and ns come from reweighting and cost nothing)."""
    from camb_gb300 import gradients
    members, _ = gradients.fd_members(ps, 1e-4)
    nth = os.cpu_count() or 1
    structs = [m.to_struct() for m in members]
    cpu_reference_batch(structs[:nth], nth)
    t = cpu_reference_batch(structs, nth)
    return {"value": len(ps) / t, "unit": "gradients/s", "cores": nth,
            "sample": f"{len(ps)} gradients ({len(structs)} cosmologies), one cosmology per thread"}


def gradient_checks(ps, g):
    """On the first draws of the gradient batch (outside the timed call): the largest
    disagreement of the GPU's central differences with the oracle's (same perturbed
    cosmologies, sampled l, TT/EE/TE, relative to each gradient's peak over l) per
    parameter, and the finite-difference noise as the disagreement of relative steps 1e-4
    and 3e-4 (GPU, same statistic; median and largest over l)."""
    import copy
    from camb_gb300 import _lib, gradients
    from oracle import oracle as orc
    vs_oracle, noise = {}, {}
    _, g3 = gradients.cl_gradients(ps, rel_step=3e-4)
    for name in gradients.EVOLVED:
        j = gradients.PARAMS.index(name)
        worst, med, mx = 0.0, 0.0, 0.0
        for i, p in enumerate(ps):
            v = gradients.get_param(p, name)
            h = 1e-4 * abs(v)
            icl = []
            for sgn in (1.0, -1.0):
                q = copy.deepcopy(p)
                gradients.set_param(q, name, v + sgn * h)
                T = _lib.Tables(q.to_struct())
                icl.append(orc.cls(T, orc.los(T, orc.evolve_sources(T))))
            ls = T.ls
            ref = (icl[0] - icl[1]) / (2 * h)
            for cg, cr in [(0, 0), (1, 1), (3, 2)]:
                peak = np.max(np.abs(ref[:, cr]))
                worst = max(worst, float(np.max(np.abs(g[i, j][ls, cg] - ref[:, cr])) / peak))
                d = np.abs(g[i, j][ls, cg] - g3[i, j][ls, cg]) / np.max(np.abs(g[i, j][ls, cg]))
                med, mx = max(med, float(np.median(d))), max(mx, float(d.max()))
        vs_oracle[name] = worst
        noise[name] = {"median": med, "max": mx}
    return {"max_rel_disagreement_vs_oracle_fd": vs_oracle,
            "fd_noise_step_1e-4_vs_3e-4": noise,
            "checked_draws": len(ps)}


def lensed_batch(n, lmax=2500, seed=5000, mnu_max=0.2):
    """The batched lensed configuration: n lensed draws (lmax 2500 + 200 margin) resident
    on the device.  On grids shared by the batch (cambgpu_batch_prepare_shared) the
    pipeline runs with the FP64 projection, the FP32 (mixed) projection and the split hi/lo
    BF16 tensor-core projection; each form's device time per stage and the lensed C_l error
    of the mixed and tensor forms against FP64 per l band are reported.  The same draws on
    their own grids (cambgpu_batch_prepare, FP64) give the shift that sharing the grids
    causes, stated separately."""
    from camb_gb300 import _lib
    lib = _lib.load()
    ps = workload(n, lmax, seed=seed, mnu_max=mnu_max)
    for p in ps:
        p.do_lensing = 1
        p.max_l = lmax + 200
        p.max_eta_k = 2.5 * p.max_l
    arr = (_lib.CambGpuParams * n)(*ps)
    L = lmax + 200

    def spectra():
        unl = np.zeros((n, L + 1, 4))
        len_ = np.zeros((n, L + 1, 4))
        pot = np.zeros((n, L + 1, 3))
        lml = np.zeros(n, dtype=np.int32)
        _lib.check(lib.cambgpu_batch_spectra_from_transfer(None, None, None, None, L, _lib.dptr(unl), _lib.dptr(len_),
                                                           _lib.dptr(pot), _lib.iptr(lml)))
        return len_, pot

    def run_forms(forms, shared):
        out, ms_form = {}, {}
        t0 = time.perf_counter()
        if shared:
            nchi = C.c_int()
            _lib.check(lib.cambgpu_batch_prepare_shared(arr, n, C.byref(nchi)))
        else:
            _lib.check(lib.cambgpu_batch_prepare(arr, n))
        prep = time.perf_counter() - t0
        for mode in forms:
            _lib.check(lib.cambgpu_set_precision(mode))
            ms = np.zeros(3)
            _lib.check(lib.cambgpu_batch_run(_lib.dptr(ms)))  # warm-up (graph capture on the next)
            _lib.check(lib.cambgpu_batch_run(_lib.dptr(ms)))
            ms_form[mode] = ms.copy()
            out[mode] = spectra()
        lib.cambgpu_batch_release()
        return out, ms_form, prep, (nchi.value if shared else None)

    sh, ms_sh, prep_sh, nchi = run_forms((0, 1, 2), True)
    nat, ms_nat, prep_nat, _ = run_forms((0,), False)
    _lib.check(lib.cambgpu_set_precision(1))
    bands = [(2, 100), (100, 500), (500, 1000), (1000, 1500), (1500, 2000), (2000, lmax)]

    def band_err(got, ref):
        err = {}
        for lo, hi in bands:
            sl = slice(lo, hi + 1)
            g, r = got[0][:, sl], ref[0][:, sl]
            err[f"{lo}-{hi}"] = {"TT": float(np.max(np.abs(g[..., 0] / r[..., 0] - 1))),
                                 "EE": float(np.max(np.abs(g[..., 1] / r[..., 1] - 1))),
                                 "BB": float(np.max(np.abs(g[..., 2] / r[..., 2] - 1))),
                                 "TE_over_sqrt_TTEE": float(np.max(np.abs(g[..., 3] - r[..., 3]) /
                                                                   np.sqrt(r[..., 0] * r[..., 1]))),
                                 "PP": float(np.max(np.abs(got[1][:, sl, 0] / ref[1][:, sl, 0] - 1)))}
        return err

    names = {0: "fp64", 1: "mixed_fp32", 2: "tensor_bf16x3"}
    stage = {names[k]: {"ode": v[0], "spline_los": v[1], "cls_interp_lens": v[2]} for k, v in ms_sh.items()}
    # the CPU restatement on the first draws, each on its own grids, one cosmology per thread
    nth = os.cpu_count() or 1
    sample = ps[:2 * nth]
    t_cpu = cpu_reference_batch(sample, nth, lensed=True)
    cpu = {"value": len(sample) / t_cpu, "unit": "cosmologies/s", "cores": nth,
           "sample": f"the batch's first {len(sample)} draws on their own grids, one cosmology per thread, host "
                     f"tables + ODE + LOS + C_l + interpolation + lensing"}
    return {"config": {"workload": f"{n} seeded draws (fiducial LCDM +-5%, mnu 0-{mnu_max:g} eV), lensed "
                                   f"TT/EE/BB/TE and phi-phi to lmax={lmax} (+200 margin), on grids shared by "
                                   f"the batch ({nchi} comoving-distance nodes)", "batch": n},
            "prepare_s": {"shared": prep_sh, "native": prep_nat}, "stage_ms_shared_grids": stage,
            "stage_ms_native_grids_fp64": {"ode": ms_nat[0][0], "spline_los": ms_nat[0][1],
                                           "cls_interp_lens": ms_nat[0][2]},
            "cosmologies_per_s": {names[k]: n / (sum(v) * 1e-3) for k, v in ms_sh.items()},
            "cpu_baseline": cpu,
            "projection_ms": {names[k]: v[1] for k, v in ms_sh.items()},
            "tensor_vs_fp64_same_grids_per_l_band": band_err(sh[2], sh[0]),
            "mixed_vs_fp64_same_grids_per_l_band": band_err(sh[1], sh[0]),
            "shared_vs_native_grids_fp64_per_l_band": band_err(sh[0], nat[0])}


def workload(n, lmax, seed, mnu_max=0.2):
    """The batch's seeded draws (camb_gb300.workload.batch_draws)."""
    from camb_gb300.workload import batch_draws
    return batch_draws(n, lmax, seed, mnu_max)


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, index=0):
        self.samples, self.index, self.proc = [], index, None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(s[0]) for s in self.samples if len(s) >= 6 and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) >= 6 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) >= 6 for i in range(4)
                          if s[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def cpu_reference(params, nthreads, keep=None):
    """Reference CPU path on the host cores: host tables + restated ODE/LOS/C_l.  With
    keep=list, appends (sampled ls, C_l at those ls) of each cosmology."""
    from camb_gb300 import _lib
    from oracle import oracle as orc
    t0 = time.perf_counter()
    for p in params:
        T = _lib.Tables(p)
        src = orc.evolve_sources(T, nthreads)
        d = orc.los(T, src, nthreads)
        icl = orc.cls(T, d)
        if keep is not None:
            keep.append((T.ls, icl))
    return time.perf_counter() - t0


def cpu_reference_batch(params, nthreads, lensed=False):
    """The same CPU path with the cosmologies spread over the host threads, each
    cosmology on one thread (the batch-parallel form, beside the reference's own
    OpenMP-over-k parallelism of cpu_reference).  The ctypes calls release the GIL.  With
    lensed=True also the interpolation to every l and the lensing of the C_l."""
    from concurrent.futures import ThreadPoolExecutor
    from camb_gb300 import _lib
    from oracle import oracle as orc
    orc.load()

    def one(p):
        T = _lib.Tables(p)
        icl = orc.cls(T, orc.los(T, orc.evolve_sources(T, 1), 1))
        if lensed:
            allc = orc.interpolate_cls(T.ls, icl, T.view.cl_template_scale)
            orc.lens_cls(allc[:, :4], T.ls, p.max_l, lens_accuracy_boost=T.view.lens_accuracy_boost)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(nthreads) as ex:
        list(ex.map(one, params))
    return time.perf_counter() - t0


def cpu_baseline_rate(args, rank, steps):
    """Cosmologies/s of the CPU path on all host cores in both parallel forms, on the
    batch's first draws (same seed and distribution as the GPU arm): OpenMP over k, one
    cosmology at a time (cpu_sample draws per step), and one cosmology per thread (two
    draws per thread per step).  The faster form is the baseline."""
    nth = os.cpu_count() or 1
    ps = workload(max(args.cpu_sample, 2 * nth), args.lmax, seed=1000 + rank, mnu_max=args.mnu_max)
    pk = ps[:args.cpu_sample]
    cpu_reference(pk[:1], nth)
    t_k = statistics.mean([cpu_reference(pk, nth) for _ in range(steps)])
    pb = ps[:2 * nth]
    cpu_reference_batch(pb[:nth], nth)
    t_b = statistics.mean([cpu_reference_batch(pb, nth) for _ in range(steps)])
    forms = {"openmp_over_k": {"value": len(pk) / t_k, "draws_per_step": len(pk)},
             "cosmology_per_thread": {"value": len(pb) / t_b, "draws_per_step": len(pb)}}
    best = max(forms, key=lambda f: forms[f]["value"])
    return {"value": forms[best]["value"], "unit": "cosmologies/s", "cores": nth, "kind": "port",
            "form": best, "forms": forms,
            "sample": f"the batch's first {forms[best]['draws_per_step']} draws per step, host tables + ODE + LOS + "
                      f"C_l, {'one cosmology per thread' if best == 'cosmology_per_thread' else 'OpenMP over k'}",
            "ms_per_step": (t_b if best == "cosmology_per_thread" else t_k) * 1e3}


def accuracy_vs_fp64(params, ref, lmax):
    """max |dC_l/C_l| (TT, EE) and max |dTE|/sqrt(TT EE) over the sampled l of the GPU
    C_l (through cambgpu_get_results_batch) against the FP64 CPU restatement."""
    from camb_gb300 import _lib
    lib = _lib.load()
    n = len(params)
    arr = (_lib.CambGpuParams * n)(*params)
    cls = np.zeros((n, lmax + 1, 4))
    st = np.zeros(n, dtype=np.int32)
    _lib.check(lib.cambgpu_get_results_batch(arr, n, lmax, _lib.dptr(cls), _lib.iptr(st)))
    tt = ee = te = 0.0
    for i, (ls, icl) in enumerate(ref):
        m = (ls >= 2) & (ls <= lmax)
        g, r = cls[i][ls[m]], icl[m]
        tt = max(tt, float(np.max(np.abs(g[:, 0] / r[:, 0] - 1))))
        ee = max(ee, float(np.max(np.abs(g[:, 1] / r[:, 1] - 1))))
        te = max(te, float(np.max(np.abs(g[:, 3] - r[:, 2]) / np.sqrt(r[:, 0] * r[:, 1]))))
    return {"vs": "FP64 CPU restatement, same draws as cpu_baseline", "max_rel_TT": tt, "max_rel_EE": ee,
            "max_TE_over_sqrt_TTEE": te}


def single_configs(nthreads):
    """One cosmology per configuration of the benchmark suite, GPU (C ABI, host buffers)
    against the CPU restatement on the host cores, both with their host tables: the
    plain massless lmax 1000 case; one 0.06 eV neutrino with lensed TT/EE/BB/TE and the
    lensing potential to lmax 2500, at max_eta_k = 2.5 (lmax + 200) and at the reference's
    automatic lens_potential_accuracy 4 (max_eta_k = 72000, linear lensing); that
    cosmology's matter transfer functions to kmax = 10 h/Mpc at z = 0 (computed without the
    CMB); and a run that wants the CMB and high-precision transfer functions together."""
    from camb_gb300 import _lib
    from oracle import oracle as orc
    lib = _lib.load()

    def base(lmax, lensing, mnu):
        p = _lib.default_params()
        p.H0, p.ombh2, p.omch2, p.optical_depth, p.As, p.ns = 67.5, 0.022, 0.122, 0.06, 2.1e-9, 0.965
        p.nnu = 3.046
        p.mnu, p.num_massive_neutrinos = mnu, 1
        p.do_lensing = 1 if lensing else 0
        p.max_l = lmax + (200 if lensing else 0)
        p.max_eta_k = 2.5 * p.max_l
        return p

    def gpu_cmb(p):
        n = p.max_l + 1
        unl = np.zeros((n, 4))
        lens = np.zeros((n, 4)) if p.do_lensing else None
        pot = np.zeros((n, 3)) if p.do_lensing else None
        st = (C.c_int * 1)()
        lml = (C.c_int * 1)()
        _lib.check(lib.cambgpu_get_spectra_batch(C.byref(p), 1, p.max_l, _lib.dptr(unl),
                                                 _lib.dptr(lens) if lens is not None else None,
                                                 _lib.dptr(pot) if pot is not None else None, lml, st))

    def cpu_cmb(p):
        T = _lib.Tables(p)
        icl = orc.cls(T, orc.los(T, orc.evolve_sources(T, nthreads), nthreads))
        allc = orc.interpolate_cls(T.ls, icl, T.view.cl_template_scale)
        if p.do_lensing:
            orc.lens_cls(allc[:, :4], T.ls, p.max_l)

    def transfer_params():
        p = base(2500, False, 0.06)
        p.want_cls, p.want_transfer, p.transfer_high_precision = 0, 1, 1
        p.transfer_kmax = 10 * p.H0 / 100
        p.num_transfer_redshifts = 1
        p.transfer_redshifts[0] = 0.0
        return p

    def gpu_tr(p):
        tr = np.zeros((1, 1, 4096, 13), dtype=np.float32)
        nq = (C.c_int * 1)()
        s8 = np.zeros(1)
        sv = np.zeros(1)
        st = (C.c_int * 1)()
        _lib.check(lib.cambgpu_get_transfer_batch(C.byref(p), 1, 4096, tr.ctypes.data_as(C.POINTER(C.c_float)), nq,
                                                  _lib.dptr(s8), _lib.dptr(sv), st))
        return s8[0]

    def cpu_tr(p):
        T = _lib.Tables(p)
        return orc.sigma8(T, orc.evolve_transfer(T, nthreads))[0][0]

    def timed(f, p, reps=2):
        f(p)
        t0 = time.perf_counter()
        for _ in range(reps):
            r = f(p)
        return (time.perf_counter() - t0) / reps * 1e3, r

    out = {}
    lpa4 = base(2500, True, 0.06)
    lpa4.max_eta_k = 72000.0  # the reference's automatic lens_potential_accuracy 4 at lmax 2500
    for name, p in [("lmax1000_unlensed_massless", base(1000, False, 0.0)),
                    ("lmax2500_lensed_mnu0.06", base(2500, True, 0.06)),
                    ("lmax2500_lensed_mnu0.06_max_eta_k72000", lpa4)]:
        g, _ = timed(gpu_cmb, p)
        c, _ = timed(cpu_cmb, p, reps=1)
        out[name] = {"gpu_ms": g, "cpu_ms": c, "cpu_threads": nthreads}
    p = transfer_params()
    g, s8g = timed(gpu_tr, p)
    c, s8c = timed(cpu_tr, p, reps=1)
    out["transfer_kmax10h_mnu0.06_z0"] = {"gpu_ms": g, "cpu_ms": c, "cpu_threads": nthreads, "sigma8_gpu": s8g,
                                           "sigma8_cpu": s8c}

    # the CMB and high-precision transfer functions in one run (set_matter_power with the CMB
    # on: z = 3.1, 0.17, 0 to k = 1.2 /Mpc, testPowers' run): the GPU's single launch through
    # the C ABI against the CPU restatement of the reference's single evolution
    def both_params():
        p = base(2500, False, 0.07)
        p.want_transfer, p.transfer_high_precision, p.transfer_kmax = 1, 1, 1.2
        p.num_transfer_redshifts = 3
        for i, z in enumerate((3.1, 0.17, 0.0)):
            p.transfer_redshifts[i] = z
        return p

    def gpu_both(p):
        n = p.max_l + 1
        unl = np.zeros((n, 4))
        tr = np.zeros((1, 3, 1024, 13), dtype=np.float32)
        nq = (C.c_int * 1)()
        s8 = np.zeros(3)
        sv = np.zeros(3)
        st = (C.c_int * 1)()
        lml = (C.c_int * 1)()
        _lib.check(lib.cambgpu_get_results_with_transfers(C.byref(p), 1, p.max_l, _lib.dptr(unl), None, None, lml, 1024,
                                                          tr.ctypes.data_as(C.POINTER(C.c_float)), nq, _lib.dptr(s8),
                                                          _lib.dptr(sv), st))
        return s8[2]

    def cpu_both(p):
        T = _lib.Tables(p)
        src, tr = orc.evolve_combined(T, nthreads)
        orc.interpolate_cls(T.ls, orc.cls(T, orc.los(T, src, nthreads)), T.view.cl_template_scale)
        return orc.sigma8(T.transfer_view(), tr)[0][2]

    p = both_params()
    g, s8g = timed(gpu_both, p)
    c, s8c = timed(cpu_both, p, reps=1)
    out["lmax2500_mnu0.07_with_transfers_3z_kmax1.2"] = {"gpu_ms": g, "cpu_ms": c, "cpu_threads": nthreads,
                                                         "sigma8_z0_gpu": s8g, "sigma8_z0_cpu": s8c}
    return out


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    return rank, world


def barrier_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, rank, world):
    if rank != 0:
        return
    cb = cpu_baseline_rate(args, rank, args.steps)
    v = cb["value"]
    line = {"impl": "reference", "metric": METRIC,
            "value": v,
            "unit": "cosmologies/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": cb["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic seeded draws",
            "config": {"workload": f"batch of {args.batch} seeded draws (fiducial LCDM +-5%, mnu 0-{args.mnu_max:g} "
                                   f"eV), unlensed TT/EE/TE to lmax={args.lmax}, max_eta_k={2.5 * args.lmax:g}",
                       "sample": cb["sample"] + " (CPU time bounded)", "forms": cb["forms"]},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "form")},
            "e2e": {"value": v, "unit": "cosmologies/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.lensed_batch:
        print(json.dumps(lensed_batch(args.lensed_batch, args.lmax, mnu_max=args.mnu_max)))
        return
    rank, world = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    from camb_gb300 import _lib
    lib = _lib.load()
    torch.cuda.init()
    if args.team:
        _lib.check(lib.cambgpu_set_ode_team(args.team))
    B = args.batch
    ps = workload(B, args.lmax, seed=1000 + rank, mnu_max=args.mnu_max)
    arr = (_lib.CambGpuParams * B)(*ps)
    tuned = None
    if not args.team and not args.no_autotune:
        best = (C.c_int * 4)()
        times = np.zeros(16)
        _lib.check(lib.cambgpu_autotune_ode(arr, B, best, _lib.dptr(times)))
        sched = [0] * 11 + [1] * 5
        tried = [i for i in range(16) if times[i] > 0]
        tuned = {"team": best[0], "queue_order": best[1], "blocks_per_sm_cap": best[3],
                 "schedule": "static stride" if sched[min(tried, key=lambda i: times[i])] else "queue counter",
                 "candidates": "team,order,blocks-per-SM cap,schedule: 32,0,0,0 1,0,0,0 1,2,0,0 2,2,0,0 1,3,2,0 "
                               "1,2,2,0 2,2,2,0 1,1,2,0 6,0,0,0 7,2,0,0 7,3,0,0 7,2,0,1 7,3,0,1 7,4,0,1 "
                               "1,4,0,1 2,4,0,1",
                 "candidate_ode_ms": [round(x, 2) for x in times[:16]]}
    # ---- device-resident pipeline, FP64 form then mixed precision ----
    _lib.check(lib.cambgpu_batch_prepare(arr, B))

    def resident(mode):
        _lib.check(lib.cambgpu_set_precision(mode))
        ms = np.zeros(3)
        for _ in range(args.warmup):
            _lib.check(lib.cambgpu_batch_run(_lib.dptr(ms)))
        stage = np.zeros(3)
        evals = 0
        lib.cambgpu_kernel_launches(1)
        barrier(world)
        torch.cuda.synchronize()
        with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                _lib.check(lib.cambgpu_batch_run(_lib.dptr(ms)))
                stage += ms
                evals += lib.cambgpu_last_ode_evals()
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        launches = lib.cambgpu_kernel_launches(1)
        barrier(world)
        step_ms = barrier_max(stage.sum() / args.steps, world)
        out = np.zeros((B, args.lmax + 1, 4))
        _lib.check(lib.cambgpu_batch_fetch(args.lmax, _lib.dptr(out)))
        return dict(step_ms=step_ms, stage=stage / args.steps, evals=evals / args.steps, launches=launches,
                    wall=wall, clocks=clk.summary(), cls=out)

    plain = resident(0)
    mixed = resident(args.precision)
    lib.cambgpu_batch_release()
    run = mixed
    value = world * B / (run["step_ms"] * 1e-3)
    # C_l error of the timed form against the FP64 form over the whole batch
    sl = slice(2, args.lmax + 1)
    a, r = run["cls"][:, sl], plain["cls"][:, sl]
    batch_err = {"vs": f"FP64 GPU form, all {B} draws, 2<=l<={args.lmax}",
                 "max_rel_TT": float(np.max(np.abs(a[..., 0] / r[..., 0] - 1))),
                 "max_rel_EE": float(np.max(np.abs(a[..., 1] / r[..., 1] - 1))),
                 "max_TE_over_sqrt_TTEE": float(np.max(np.abs(a[..., 3] - r[..., 3]) / np.sqrt(r[..., 0] * r[..., 1])))}
    # ---- end to end through the C ABI (host params -> host C_l), timed form ----
    cls = np.zeros((B, args.lmax + 1, 4))
    st = np.zeros(B, dtype=np.int32)
    _lib.check(lib.cambgpu_get_results_batch(arr, B, args.lmax, _lib.dptr(cls), _lib.iptr(st)))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _lib.check(lib.cambgpu_get_results_batch(arr, B, args.lmax, _lib.dptr(cls), _lib.iptr(st)))
    single_s = barrier_max((time.perf_counter() - t0) / args.steps, world)
    host_ms = np.zeros(4)
    lib.cambgpu_last_host_timings(_lib.dptr(host_ms))
    xfer = (C.c_longlong * 2)()
    lib.cambgpu_last_transfer_bytes(xfer)
    # the same calls as a stream of batches in its steady state: step k+1's host tables are
    # built on a host thread while the device runs step k (cambgpu_prepare_tables /
    # _get_spectra_prepared, as camb_gb300.get_results_stream does), the first step's
    # before the timer and one batch beyond the last inside it; every step uploads its
    # tables and reads back its C_l
    first = prepare_first(lib, arr, B)
    barrier(world)
    t0 = time.perf_counter()
    stream_steps(lib, arr, B, args.steps, args.lmax, cls, st, first=first)
    e2e_s = barrier_max((time.perf_counter() - t0) / args.steps, world)
    stage, evals, launches, wall, clk = run["stage"], run["evals"], run["launches"], run["wall"], run["clocks"]
    step_ms = run["step_ms"]
    # ---- roofline of the dominant kernel (ODE, FP64 pipe) ----
    tf = C.c_double()
    _lib.check(lib.cambgpu_probe_fp64_tflops(C.byref(tf)))
    ode_ms = stage[0]
    evals_step = evals
    # FP64 flops per right-hand-side evaluation, stage combinations and error norm
    # included: 2*DFMA + DMUL + DADD thread instructions per evaluation counted by ncu on
    # a 32-draw case of this workload (mnu 0-0.2 eV, lmax 2500)
    flops_per_eval = float(FLOPS_PER_EVAL)
    achieved = flops_per_eval * evals_step / (ode_ms * 1e-3) / 1e12
    ode_team = args.team or (tuned["team"] if tuned else 0)
    ode_order = tuned["queue_order"] if tuned else -1
    traffic, traffic_src = ODE_TRAFFIC.get((ode_team, ode_order),
                                           (None, f"no ncu capture of team {ode_team}, order {ode_order}"))
    if tuned and traffic:
        traffic_src += f"; the timed launches use the {tuned['schedule']} schedule"
    prec = {0: "FP64 throughout",
            1: "FP64 ODE, source k-spline, C_l integral; FP32 line-of-sight projection with FP64 chunk sums"}
    line = {"metric": METRIC, "value": value,
            "unit": "cosmologies/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == 0 else "f64+f32", "data": "synthetic seeded draws",
            "config": {"precision": prec[args.precision],
                       "workload": f"batch of {B} seeded draws (fiducial LCDM +-5%, mnu 0-{args.mnu_max:g} eV), "
                                   f"unlensed TT/EE/TE to lmax={args.lmax}, max_eta_k={2.5 * args.lmax:g}",
                       "global_batch": B * world, "per_gpu_batch": B, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (per-cosmology tables ~3 MB x batch)",
                       "ode_autotune": tuned,
                       "stage_ms": {"ode": stage[0], "spline_los": stage[1], "cls_interp_lens": stage[2]}},
            "fp64_form": {"value": world * B / (plain["step_ms"] * 1e-3), "ms_per_step": plain["step_ms"],
                          "stage_ms": {"ode": plain["stage"][0], "spline_los": plain["stage"][1],
                                       "cls_interp_lens": plain["stage"][2]}},
            "accuracy_vs_fp64_gpu": batch_err,
            "e2e": {"value": world * B / e2e_s, "unit": "cosmologies/s", "h2d_bytes_per_step": int(xfer[0]),
                    "d2h_bytes_per_step": int(xfer[1]),
                    "form": "stream of batches in steady state: host tables of the next batch built while the "
                            "device runs this one (the first batch's before the timer, one beyond the last "
                            "inside it)",
                    "single_call_value": world * B / single_s,
                    "last_call_ms": {"host_tables": host_ms[0], "staging": host_ms[1], "device": host_ms[2],
                                     "fetch": host_ms[3]}},
            "gpu_launches": int(launches),
            "roofline": {"bound": "fp64", "kernel": "ode_thread_kernel", "achieved": achieved, "peak": tf.value,
                         "unit": "TFLOP/s", "frac": achieved / tf.value, "traffic": traffic,
                         "peak_source": "DFMA-chain probe measured in this run (MEASURED_PEAKS.json has no FP64)",
                         "frac_of_nominal_fp64": achieved / NOMINAL_FP64_TFLOPS,
                         "nominal_fp64_tflops": NOMINAL_FP64_TFLOPS,
                         "flops_per_eval": flops_per_eval, "evals_per_step": evals_step,
                         "traffic_source": traffic_src,
                         "dram_gbs": traffic / (ode_ms * 1e-3) / 1e9 if traffic else None,
                         "dram_frac_of_measured_copy":
                             traffic / (ode_ms * 1e-3) / 1e9 / hbm_peak() if traffic else None,
                         "flops_source": "ncu 2 DFMA + DMUL + DADD thread instructions per evaluation, kernel case "
                                         "thread32 (profiles/ode_thread_kernel_batch32_lmax2500.md)",
                         "reading": "the seven stage rows of the resident modes exceed L1 and L2 and stream through "
                                    "DRAM; a warp issues one FP64 instruction per 64 cycles and two warps per "
                                    "sub-partition cannot cover that latency (profiles/fp64_issue_model.md)"},
            "clocks": clk, "wall_s_timed": wall}
    if rank == 0:
        nth = os.cpu_count() or 1
        # the batch's first cpu_sample draws: the same cosmologies the reference arm times
        cps = workload(args.cpu_sample, args.lmax, seed=1000 + rank, mnu_max=args.mnu_max)
        cpu_reference(cps[:1], nth)
        ref = []
        t = cpu_reference(cps, nth, keep=ref)
        line["accuracy"] = accuracy_vs_fp64(cps, ref, args.lmax)  # timed form vs the FP64 CPU restatement
        line["single_cosmology_configs"] = single_configs(nth)
        line["gradients"] = gradient_rate()
        # the batched lensed configuration's projections on grids shared by the batch (the
        # full 1024-draw case: bench.py --lensed-batch 1024)
        lb = lensed_batch(256, args.lmax, mnu_max=args.mnu_max)
        line["shared_grid_projections_lensed_256"] = {
            "projection_ms": lb["projection_ms"], "cosmologies_per_s": lb["cosmologies_per_s"],
            "cpu_baseline": lb["cpu_baseline"],
            "tensor_vs_fp64_same_grids_max": {k: max(b[k] for b in lb["tensor_vs_fp64_same_grids_per_l_band"].values())
                                               for k in ("TT", "EE", "BB", "TE_over_sqrt_TTEE", "PP")},
            "shared_vs_native_grids_fp64_max": {k: max(b[k] for b in
                                                       lb["shared_vs_native_grids_fp64_per_l_band"].values())
                                                 for k in ("TT", "EE", "BB", "TE_over_sqrt_TTEE", "PP")},
            "workload": lb["config"]["workload"]}
        plain = plain_form_rate(mnu_max=args.mnu_max)
        line["batched_vs_plain_gpu"] = {
            "plain_fp64_gpu_cosmologies_per_s": plain,
            "plain_form": "one cosmology per blocking C-ABI call, FP64 throughout, same workload, host tables included",
            "ratio_value": line["value"] / plain, "ratio_e2e": line["e2e"]["value"] / plain}
        cb = cpu_baseline_rate(args, rank, 2)
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample", "form", "forms")}
        print(json.dumps(line))


if __name__ == "__main__":
    main()
