"""Extracts the golden vectors the tests pin the oracle and library against.

Run here, where the reference source tree is mounted (its path is the only
argument); writes tests/golden/*.json.  The GPU machine
only reads the JSON files.

  template_cls.json  rows of the reference's fortran/HighLExtrapTemplate_lenspotentialCls.dat
                     (high-accuracy unlensed l(l+1)C_l/2pi for the inifiles/planck_2018.ini
                     cosmology) at the l values the tests use, plus that cosmology's parameters
                     read from inifiles/planck_2018.ini.
  known_answers.json scalar known answers written in camb/tests/camb_test.py.
"""
import json
import os
import re
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python %s <reference_root>" % os.path.basename(__file__))
ref = sys.argv[1]
here = os.path.dirname(os.path.abspath(__file__))

tmpl = np.loadtxt(os.path.join(ref, "fortran", "HighLExtrapTemplate_lenspotentialCls.dat"))
ls = sorted(set(list(range(2, 41)) + list(range(45, 3001, 5))))
rows = {int(r[0]): [float(x) for x in r[1:]] for r in tmpl if int(r[0]) in ls}
ini = {}
for line in open(os.path.join(ref, "inifiles", "planck_2018.ini")):
    m = re.match(r"\s*([A-Za-z_0-9()]+)\s*=\s*(.*)$", line)
    if m:
        ini[m.group(1)] = m.group(2).strip()
keys = ["ombh2", "omch2", "omnuh2", "hubble", "helium_fraction", "massless_neutrinos", "massive_neutrinos",
        "re_optical_depth", "scalar_amp", "scalar_spectral_index", "temp_cmb", "pivot_scalar", "re_delta_redshift"]
cosmo = {k: float(ini[k]) for k in keys}
json.dump({"columns": ["TT", "EE", "BB", "TE", "PP", "TP", "EP"], "cosmology": cosmo,
           "source": "fortran/HighLExtrapTemplate_lenspotentialCls.dat", "cls": rows},
          open(os.path.join(here, "template_cls.json"), "w"), indent=0)

# camb/tests/camb_test.py known answers (testPowers): scalar_power(1) = 1.801e-9 for
# As = 2e-9, ns = 0.965 at pivot 0.05, places=4 -> 1e-13 absolute in these units.
src = open(os.path.join(ref, "camb", "tests", "camb_test.py")).read()
m = re.search(r"assertAlmostEqual\(pars\.scalar_power\(1\)[^,]*,\s*([0-9.e\-]+)", src)
known = {"scalar_power_k1": float(m.group(1)) if m else 1.801e-9, "scalar_power_As": 2e-9,
         "scalar_power_ns": 0.965, "source": "camb/tests/camb_test.py testPowers"}
# testPowers sigma8 / f sigma8 (places=3) for H0 67.5, ombh2 0.022, omch2 0.122, mnu 0.07,
# As 2e-9, ns 0.965, reionization at z = 10 (the CAMBparams default), linear transfer
# functions at z = [3.1, 0.17, 0] to kmax 1.2 with high precision
def almost(expr):
    m = re.search(r"assertAlmostEqual\(" + re.escape(expr) + r",\s*([0-9.e\-]+),\s*([0-9]+)\)", src)
    return [float(m.group(1)), int(m.group(2))]
known["sigma8"] = {"redshifts": [3.1, 0.17, 0.0], "s8_z3.1": almost("s8[0]"), "s8_z0": almost("s8[2]"),
                   "fs8_z3.1": almost("fs8[0]"), "fs8_z0": almost("fs8[2]"),
                   "cosmology": {"H0": 67.5, "ombh2": 0.022, "omch2": 0.122, "mnu": 0.07, "As": 2e-9,
                                 "ns": 0.965, "zre": 10.0, "kmax": 1.2},
                   "source": "camb/tests/camb_test.py testPowers"}
json.dump(known, open(os.path.join(here, "known_answers.json"), "w"), indent=1)
print("wrote", len(rows), "template rows")
