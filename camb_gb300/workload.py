"""Seeded parameter draws of the batched benchmark workload.

Each draw is the fiducial flat LCDM cosmology (H0 67.5, ombh2 0.022, omch2 0.122,
tau 0.06, As 2.1e-9, ns 0.965, N_eff 3.046) with each of ombh2, omch2, H0, tau, As,
ns scaled by a factor uniform in [0.95, 1.05], plus one massive neutrino eigenstate
of mass uniform in [0, mnu_max] eV, unlensed scalar C_l to lmax with
max_eta_k = 2.5 lmax (the reference's set_for_lmax default, camb/model.py:1018-1063).
"""
import numpy as np

from . import _lib


def batch_draws(n, lmax, seed, mnu_max=0.2):
    """n CambGpuParams of the workload, drawn with numpy.random.default_rng(seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        p = _lib.default_params()
        p.H0, p.ombh2, p.omch2, p.optical_depth, p.As, p.ns = 67.5, 0.022, 0.122, 0.06, 2.1e-9, 0.965
        p.nnu = 3.046
        for name in ["ombh2", "omch2", "H0", "optical_depth", "As", "ns"]:
            setattr(p, name, getattr(p, name) * (1 + 0.05 * (2 * rng.random() - 1)))
        if mnu_max > 0:
            p.mnu = mnu_max * rng.random()
            p.num_massive_neutrinos = 1
        p.max_l = lmax
        p.max_eta_k = 2.5 * lmax
        out.append(p)
    return out
