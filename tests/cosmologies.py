"""Parameter sets shared by the tests (the reference's test configurations)."""
import json
import os

import numpy as np

from camb_gb300 import _lib

HERE = os.path.dirname(os.path.abspath(__file__))


def fiducial(lmax=1000, lensing=False, **over):
    """Plain flat LCDM of the scalar-path benchmark: H0=67.5, ombh2=0.022, omch2=0.122,
    massless N_eff, tau=0.06, As=2.1e-9, ns=0.965."""
    p = _lib.default_params()
    p.H0, p.ombh2, p.omch2, p.optical_depth, p.As, p.ns = 67.5, 0.022, 0.122, 0.06, 2.1e-9, 0.965
    p.nnu = 3.046
    p.max_l = lmax
    p.do_lensing = 1 if lensing else 0
    p.max_eta_k = (lmax + (200 if lensing else 0)) * 2.5
    if lensing:
        p.max_l = lmax + 200
    for k, v in over.items():
        setattr(p, k, v)
    return p


def planck2018(lmax=1000):
    """inifiles/planck_2018.ini cosmology: one massive neutrino of 0.06 eV (the ini's
    omnuh2), N_eff = 3.046."""
    g = json.load(open(os.path.join(HERE, "golden", "template_cls.json")))["cosmology"]
    p = _lib.default_params()
    p.ombh2 = g["ombh2"]
    p.omch2 = g["omch2"]
    p.mnu = 0.06
    p.num_massive_neutrinos = 1
    p.H0 = g["hubble"]
    p.YHe = g["helium_fraction"]
    p.nnu = g["massless_neutrinos"] + g["massive_neutrinos"]
    p.optical_depth = g["re_optical_depth"]
    p.As = g["scalar_amp"]
    p.ns = g["scalar_spectral_index"]
    p.TCMB = g["temp_cmb"]
    p.max_l = lmax
    p.max_eta_k = lmax * 2.5
    return p


def draws(n, seed=1234, lmax=1000, frac=0.05, mnu_max=0.0):
    """Seeded draws, each parameter uniform in fiducial +-5% (the batch configuration);
    with mnu_max > 0 one massive eigenstate of mass uniform in [0, mnu_max] eV."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        p = fiducial(lmax)
        for name in ["ombh2", "omch2", "H0", "optical_depth", "As", "ns"]:
            setattr(p, name, getattr(p, name) * (1 + frac * (2 * rng.random() - 1)))
        if mnu_max > 0:
            p.mnu = mnu_max * rng.random()
            p.num_massive_neutrinos = 1
        out.append(p)
    return out


def template():
    g = json.load(open(os.path.join(HERE, "golden", "template_cls.json")))
    return {int(k): np.array(v) for k, v in g["cls"].items()}


def sigma8_known_answer():
    """camb_test.py testPowers cosmology for the sigma8 known answers, as a transfer-function
    run (want_cls = 0): H0 67.5, ombh2 0.022, omch2 0.122, one 0.07 eV neutrino, As 2e-9,
    ns 0.965, reionization at z = 10, transfers at z = 3.1, 0.17, 0 to kmax 1.2 /Mpc."""
    g = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))["sigma8"]
    c = g["cosmology"]
    p = _lib.default_params()
    p.H0, p.ombh2, p.omch2, p.mnu, p.num_massive_neutrinos, p.nnu = c["H0"], c["ombh2"], c["omch2"], c["mnu"], 1, 3.044
    p.As, p.ns = c["As"], c["ns"]
    p.reion_use_optical_depth, p.reion_redshift = 0, c["zre"]
    p.want_cls, p.want_transfer, p.transfer_high_precision, p.transfer_kmax = 0, 1, 1, c["kmax"]
    p.num_transfer_redshifts = len(g["redshifts"])
    for i, z in enumerate(g["redshifts"]):
        p.transfer_redshifts[i] = z
    return p, g
