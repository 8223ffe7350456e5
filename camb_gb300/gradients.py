"""Gradients dC_l/d(ombh2, omch2, H0, tau, As, ns) through the batched GPU pipeline.

Central differences, batched: every input cosmology adds two members per parameter
that enters the perturbation equations (ombh2, omch2, H0, tau) to ONE resident batch,
so the k-modes of all of them share the persistent ODE launch.  As and ns only weight
the primordial power in the C_l k-integral, so their derivatives come from the
central member's resident transfer functions without re-evolving
(power_spectra_from_transfer, camb.f90:25-58): dC_l/dAs = C_l/As exactly, and dC_l/dns
is a central difference of the primordial weight alone.

This is the finite-difference form of the gradient.  It costs 9 cosmologies per
gradient on the device; a discrete adjoint of the stepper is not part of this package.
"""
import copy

import numpy as np

from . import _lib
from .results import _ResidentBatch

PARAMS = ("ombh2", "omch2", "H0", "tau", "As", "ns")
EVOLVED = ("ombh2", "omch2", "H0", "tau")


def get_param(p, name):
    if name == "tau":
        return p.Reion.optical_depth
    if name in ("As", "ns"):
        return getattr(p.InitPower, name)
    return getattr(p, name)


def set_param(p, name, value):
    if name == "tau":
        p.Reion.set_tau(value)
    elif name in ("As", "ns"):
        setattr(p.InitPower, name, value)
    else:
        setattr(p, name, value)


def fd_members(params_list, rel_step):
    """The batch of central and perturbed members: for each input, the input itself then
    (+h, -h) for each of EVOLVED, h = rel_step * |value|.  Returns (members, steps) with
    steps[i][j] the step of EVOLVED[j] for input i."""
    members, steps = [], []
    for p in params_list:
        if get_param(p, "tau") is None or not p.Reion.use_optical_depth:
            raise ValueError("gradients need the reionization set by its optical depth")
        members.append(p)
        hs = []
        for name in EVOLVED:
            v = get_param(p, name)
            h = rel_step * abs(v)
            for sgn in (1.0, -1.0):
                q = copy.deepcopy(p)
                set_param(q, name, v + sgn * h)
                members.append(q)
            hs.append(h)
        steps.append(hs)
    return members, steps


def cl_gradients(params_list, rel_step=1e-4, lensed=False, precision=0):
    """C_l and their gradients for a list of CAMBparams.

    Returns (cls, grads): cls[n, lmax+1, 4] as CAMBdata.get_unlensed_scalar_cls (or the
    lensed spectra with lensed=True; every input must then have DoLensing) in
    l(l+1)C_l/2pi, columns TT EE BB TE; grads[n, 6, lmax+1, 4] the derivatives with
    respect to PARAMS in that order.

    `precision` is the line-of-sight arithmetic of the batch (cambgpu_set_precision;
    the caller's setting is restored afterwards).  The default is FP64: a difference
    quotient divides the C_l error by the step, so the mixed form's ~1e-6 relative
    error would become ~5e-3 of a gradient at rel_step 1e-4."""
    n = len(params_list)
    stride = 1 + 2 * len(EVOLVED)
    members, steps = fd_members(params_list, rel_step)
    lib = _lib.load()
    prev = lib.cambgpu_get_precision()
    _lib.check(lib.cambgpu_set_precision(precision))
    try:
        batch = _ResidentBatch(members)
    finally:
        lib.cambgpu_set_precision(prev)
    col = 1 if lensed else 0

    def spectra():
        out = batch.spectra()
        return out[col]

    base = spectra()
    lmax = base.shape[1] - 1
    cls = base[::stride].copy()
    grads = np.zeros((n, len(PARAMS), lmax + 1, 4))
    for j in range(len(EVOLVED)):
        plus = base[1 + 2 * j::stride]
        minus = base[2 + 2 * j::stride]
        for i in range(n):
            grads[i, j] = (plus[i] - minus[i]) / (2 * steps[i][j])
    # primordial parameters: reweight the central members' transfer functions
    centre = [members[i * stride] for i in range(n)]
    for j, name in enumerate(("As", "ns")):
        vals = [get_param(p, name) for p in centre]
        hs = [rel_step * abs(v) for v in vals]
        res = []
        for sgn in (1.0, -1.0):
            for p, v, h in zip(centre, vals, hs):
                set_param(p, name, v + sgn * h)
            res.append(spectra()[::stride].copy())
            for p, v in zip(centre, vals):
                set_param(p, name, v)
        for i in range(n):
            grads[i, len(EVOLVED) + j] = (res[0][i] - res[1][i]) / (2 * hs[i])
    return cls, grads


def cls_function():
    """A torch.autograd.Function mapping theta[n, 6] (PARAMS order, float64) applied to a
    template CAMBparams onto C_l[n, lmax+1, 4]; backward contracts the incoming gradient
    with the central-difference Jacobian formed in forward."""
    import torch

    class CMBSpectra(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta, template, rel_step=1e-4, lensed=False):
            ps = []
            for row in theta.detach().cpu().numpy():
                p = copy.deepcopy(template)
                for name, v in zip(PARAMS, row):
                    set_param(p, name, float(v))
                ps.append(p)
            cls, grads = cl_gradients(ps, rel_step=rel_step, lensed=lensed)
            ctx.save_for_backward(torch.from_numpy(grads))
            return torch.from_numpy(cls).to(theta.device)

        @staticmethod
        def backward(ctx, g):
            (grads,) = ctx.saved_tensors
            gt = torch.einsum("nplc,nlc->np", grads.to(g.device), g.to(torch.float64))
            return gt, None, None, None

    return CMBSpectra
