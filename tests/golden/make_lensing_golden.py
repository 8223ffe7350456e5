"""Golden vectors for the lensing restatement, made with the reference's own Python
lensing (camb/correlations.py lensed_cls, the full-sky Gauss-Legendre method that the
reference tests against its Fortran curved-sky code, camb_test.py:880-906).

Run here, where the reference source tree is mounted (its path is the only argument).  The input spectra are the oracle's unlensed C_l of the
fiducial lensed cosmology (H0 67.5, ombh2 0.022, omch2 0.122, massless N_eff 3.046,
tau 0.06, As 2.1e-9, ns 0.965, max_l 2700); writes tests/golden/lensing_pin.npz with
the inputs, the lensing l range, and the reference's lensed TT EE BB TE.
"""
import importlib.util
import os
import sys

import numpy as np

here = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(here, "..", ".."))
if len(sys.argv) != 2:
    sys.exit("usage: python %s <reference_root>" % os.path.basename(__file__))
ref = sys.argv[1]

from camb_gb300 import _lib  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from tests.cosmologies import fiducial  # noqa: E402

spec = importlib.util.spec_from_file_location("ref_correlations", os.path.join(ref, "camb", "correlations.py"))
corr = importlib.util.module_from_spec(spec)
spec.loader.exec_module(corr)

p = fiducial(2500, lensing=True)
T = _lib.Tables(p)
icl = orc.cls(T, orc.los(T, orc.evolve_sources(T)))
allc = orc.interpolate_cls(T.ls, icl, T.view.cl_template_scale)
max_l = p.max_l
lmax, lmax_lensed = orc.lensing_lrange(T.ls, max_l)
L = np.arange(max_l + 1, dtype=np.float64)
cls = np.zeros((max_l + 1, 4))
cls[:, 0], cls[:, 1], cls[:, 3] = allc[:, 0], allc[:, 1], allc[:, 2]
clpp = np.zeros(max_l + 1)
clpp[2:] = allc[2:, 3] * (L[2:] + 1) ** 2 / L[2:] ** 2 / (2 * np.pi)
lensed = corr.lensed_cls(cls, clpp, lmax=lmax, lmax_lensed=lmax_lensed, delta_cls=False,
                         use_lensing_template=True, low_l_ee_taper=True)
np.savez_compressed(os.path.join(here, "lensing_pin.npz"), ls=T.ls.astype(np.int32), max_l=max_l,
                    unlensed=allc[:, :4], lmax=lmax, lmax_lensed=lmax_lensed, ref_lensed=lensed,
                    source="camb/correlations.py lensed_cls(use_lensing_template=True, low_l_ee_taper=True)")
print("wrote lensing_pin.npz", lmax, lmax_lensed)
