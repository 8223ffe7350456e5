"""Converts the reference's high-L template (fortran/HighLExtrapTemplate_lenspotentialCls.dat:
unlensed l(l+1)C_l/2pi for the planck_2018.ini cosmology at high accuracy to l=8000, with
[L(L+1)]^2 C_L^phiphi/2pi) into highl_template.f64: little-endian float64 [8001][4], row l
holding TT, EE, TE, PP, rows 0 and 1 zero.  These are the four columns the reference loads
(config.f90:93-116); the library uses them for the templated C_l interpolation
(results.f90:1745-1824) and the lensing tail extension (lensing.f90:280-336).

Run where the reference tree is mounted: python tests/golden/make_template.py <reference_root>
(writes camb_gb300/data/highl_template.f64, the product's copy of the table).
"""
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python make_template.py <reference_root>")
ref = sys.argv[1]
here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "camb_gb300", "data")
rows = np.loadtxt(os.path.join(ref, "fortran", "HighLExtrapTemplate_lenspotentialCls.dat"))
LMAX = 8000
out = np.zeros((LMAX + 1, 4), dtype="<f8")
for r in rows:
    L = int(r[0])
    if L > LMAX:
        break
    out[L] = [r[1], r[2], r[4], r[5]]
assert out[LMAX, 0] > 0, "template does not reach l=8000"
out.tofile(os.path.join(here, "highl_template.f64"))
print("wrote", out.shape)
