"""CPU tests of the C_l interpolation and lensing restatement (oracle/lensing_oracle.cpp)
against the reference's own Python lensing on golden vectors, and of the templated
interpolation on inputs whose answer is known."""
import os

import numpy as np
import pytest

from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def pin():
    return np.load(os.path.join(HERE, "golden", "lensing_pin.npz"))


def test_lensing_l_range_matches_fixture(pin):
    lmax, lmax_lensed = orc.lensing_lrange(pin["ls"], int(pin["max_l"]))
    assert (lmax, lmax_lensed) == (int(pin["lmax"]), int(pin["lmax_lensed"]))


def test_lensing_restatement_matches_reference_python(pin):
    """The Fortran default (CorrFuncFullSkyApodized, uniform theta grid, sub-sampled l)
    against the reference's Gauss-Legendre full-sky lensing on the same unlensed input.
    Lensing changes TT by up to ~12% near l=2500; the two methods agree to 3e-5 of C_l
    below l=2000 and 2e-4 up to lmax_lensed (TT, EE, TE); BB, entirely lensing, to 3e-3."""
    max_l = int(pin["max_l"])
    got = orc.lens_cls(pin["unlensed"], pin["ls"], max_l)
    ref = pin["ref_lensed"]
    n = int(pin["lmax_lensed"])
    sl = slice(2, n + 1)
    tt = np.abs(got[sl, 0] / ref[sl, 0] - 1)
    ee = np.abs(got[sl, 1] / ref[sl, 1] - 1)
    bb = np.abs(got[sl, 2] / ref[sl, 2] - 1)
    te = np.abs(got[sl, 3] - ref[sl, 3]) / np.sqrt(ref[sl, 0] * ref[sl, 1])
    assert tt[:1998].max() < 3e-5 and ee[:1998].max() < 3e-5 and te[:1998].max() < 3e-5
    assert tt.max() < 2e-4 and ee.max() < 2e-4 and te.max() < 2e-4
    assert bb.max() < 3e-3
    # lensing is not a no-op: the correction itself is what is being checked
    unl = pin["unlensed"]
    assert np.max(np.abs(got[sl, 0] / unl[sl, 0] - 1)) > 0.05


def test_lensing_amplitude_check():
    pin_ = np.load(os.path.join(HERE, "golden", "lensing_pin.npz"))
    bad = np.array(pin_["unlensed"], copy=True)
    bad[:, 3] *= 1e3  # unrealistically large lensing potential (lensing.f90:205-210, 314-317)
    with pytest.raises(RuntimeError):
        orc.lens_cls(bad, pin_["ls"], int(pin_["max_l"]))


@pytest.mark.parametrize("scale", [1.0, 1.03])
def test_templated_interpolation_reproduces_template(pin, scale):
    """C_l equal to the (scaled) template at the sampled l interpolate to the template at
    every l: the spline only sees the zero difference (results.f90:1757-1808)."""
    tmpl = orc.load_template()
    ls = pin["ls"]
    lmax = int(ls[-1])

    def scaled(col):
        tl = np.arange(lmax + 1) / scale
        lo = np.clip(tl.astype(int), 1, 7999)
        frac = tl - lo
        return (1 - frac) * tmpl[lo, col] + frac * tmpl[lo + 1, col]

    want = np.stack([tmpl[: lmax + 1, c] if scale == 1.0 else scaled(c) for c in range(3)], axis=1)
    icl = np.zeros((len(ls), 6))
    icl[:, :3] = want[ls]
    icl[:, 3] = np.linspace(1e-8, 2e-8, len(ls))
    out = orc.interpolate_cls(ls, icl, scale)
    sl = slice(int(ls[0]), lmax + 1)
    assert np.max(np.abs(out[sl, :3] / want[sl] - 1)) < 1e-12
    # untemplated column: a linear function of l is reproduced by the natural spline
    assert np.allclose(out[ls, 3], icl[:, 3], rtol=1e-14)


def test_interpolation_passes_through_knots(pin):
    ls = pin["ls"]
    rng = np.random.default_rng(3)
    icl = np.abs(rng.normal(size=(len(ls), 6))) * 1e-10
    out = orc.interpolate_cls(ls, icl, 1.0)
    assert np.allclose(out[ls], icl, rtol=1e-12, atol=1e-25)
