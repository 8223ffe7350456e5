"""Parameters, mirroring the reference's camb/model.py CAMBparams for the scalar flat path.

Only what the GPU path reads is kept: cosmology (set_cosmology, model.py:641),
l range and k range (set_for_lmax, model.py:1018-1063), the power-law primordial
spectrum (initialpower.py InitialPowerLaw.set_params) and the accuracy knobs of
AccuracyParams (model.py:164; fortran/model.f90:36-104).
"""
import ctypes as C
import math

from . import _lib
from ._lib import CAMBError


class AccuracyParams:
    """Accuracy knobs (fortran/model.f90:36-104), all default 1 / True."""

    _names = ["AccuracyBoost", "lAccuracyBoost", "lSampleBoost", "IntTolBoost", "TimeStepBoost",
              "SourcekAccuracyBoost", "IntkAccuracyBoost", "BesselBoost", "BessIntBoost", "TimeSwitchBoost",
              "LimberBoost", "BackgroundTimeStepBoost", "LensingBoost"]

    def __init__(self):
        for n in self._names:
            setattr(self, n, 1.0)
        self.AccuratePolarization = True
        self.AccurateReionization = True


class InitialPowerLaw:
    """Power-law primordial spectrum (InitialPower.f90:121-144)."""

    def __init__(self):
        self.As, self.ns, self.nrun, self.pivot_scalar = 2.1e-9, 0.965, 0.0, 0.05

    def set_params(self, As=2e-9, ns=0.96, nrun=0, pivot_scalar=0.05, **kwargs):
        if kwargs.get("r"):
            raise CAMBError("tensor modes are not part of the GPU scalar path")
        self.As, self.ns, self.nrun, self.pivot_scalar = As, ns, nrun, pivot_scalar
        return self


class TanhReionization:
    """tanh reionization set from the optical depth or the redshift (reionization.f90:97-360)."""

    def __init__(self):
        self.use_optical_depth = True
        self.optical_depth = 0.06
        self.redshift = 10.0
        self.delta_redshift = 0.5

    def set_tau(self, tau, delta_redshift=None):
        self.use_optical_depth, self.optical_depth = True, tau
        if delta_redshift is not None:
            self.delta_redshift = delta_redshift
        return self

    def set_zrei(self, zrei, delta_redshift=None):
        self.use_optical_depth, self.redshift = False, zrei
        if delta_redshift is not None:
            self.delta_redshift = delta_redshift
        return self


class Recfast:
    """CAMBparams%Recomb (recombination.py Recfast): the cosmorec fudge set is built in;
    use_rosenbrock integrates the stiff early phase with the Rosenbrock method
    (recfast.f90:739-760), as the reference does by default."""

    def __init__(self):
        self.use_rosenbrock = True


class TransferParams:
    """CAMBparams%Transfer (model.f90:160-175): matter transfer function settings."""

    def __init__(self):
        self.high_precision = False
        self.kmax = 0.9
        self.k_per_logint = 0
        self.PK_redshifts = [0.0]

    @property
    def PK_num_redshifts(self):
        return len(self.PK_redshifts)


class CAMBparams:
    def __init__(self, **kwargs):
        self.H0, self.ombh2, self.omch2, self.omk = 67.5, 0.022, 0.122, 0.0
        self.TCMB, self.YHe, self.nnu = 2.7255, 0.2454, 3.044
        self.mnu, self.num_massive_neutrinos = 0.0, 1
        self.Alens = 1.0
        self.max_l, self.max_eta_k = 2500, 6250.0
        self.DoLensing = True  # model.f90:122
        self.WantTransfer = False
        self.Transfer = TransferParams()
        self.WantCls, self.WantScalars = True, True
        self.InitPower = InitialPowerLaw()
        self.Reion = TanhReionization()
        self.Recomb = Recfast()
        self.Accuracy = AccuracyParams()
        for k, v in kwargs.items():
            setattr(self, k, v)

    def set_cosmology(self, H0=67.5, ombh2=0.022, omch2=0.12, omk=0.0, mnu=0.06, nnu=3.044, YHe=None,
                      TCMB=2.7255, tau=None, Alens=1.0, num_massive_neutrinos=1, neutrino_hierarchy="degenerate",
                      **kwargs):
        """Sets the background cosmology (model.py:641).  Massive neutrinos follow the
        degenerate hierarchy (num_massive_neutrinos eigenstates of mass mnu /
        num_massive_neutrinos, model.py:700-745 and SetNeutrinoMasses); the normal and
        inverted hierarchies are not part of this path.  YHe=None keeps 0.2454 (the BBN
        value at the fiducial ombh2) rather than recomputing BBN consistency."""
        if abs(omk) > 5e-7:
            raise CAMBError("only flat models are supported")
        if neutrino_hierarchy != "degenerate":
            raise CAMBError("only the degenerate neutrino hierarchy is supported")
        if mnu < 0 or (mnu > 0 and not 1 <= num_massive_neutrinos <= 3):
            raise CAMBError("mnu must be >= 0 with 1 to 3 massive eigenstates")
        self.H0, self.ombh2, self.omch2, self.omk = H0, ombh2, omch2, omk
        self.nnu = nnu
        self.mnu, self.num_massive_neutrinos = mnu, num_massive_neutrinos
        if YHe is not None:
            self.YHe = YHe
        self.TCMB, self.Alens = TCMB, Alens
        if tau is not None:
            self.Reion.optical_depth = tau
        return self

    def set_accuracy(self, AccuracyBoost=1.0, lSampleBoost=1.0, lAccuracyBoost=1.0, DoLateRadTruncation=True,
                     min_l_logl_sampling=None):
        """model.py set_accuracy: the overall accuracy knobs (Accuracy.AccuracyBoost,
        lSampleBoost, lAccuracyBoost).  The late radiation truncation is always on in this
        path and the log-l sampling threshold keeps its default."""
        if not DoLateRadTruncation:
            raise CAMBError("DoLateRadTruncation = False is not part of the GPU path")
        if min_l_logl_sampling:
            raise CAMBError("min_l_logl_sampling is not part of the GPU path")
        self.Accuracy.AccuracyBoost = AccuracyBoost
        self.Accuracy.lSampleBoost = lSampleBoost
        self.Accuracy.lAccuracyBoost = lAccuracyBoost
        return self

    def set_dark_energy(self, w=-1.0, cs2=1.0, wa=0, use_tabulated_w=False, wde_a_array=None, wde_w_array=None,
                        dark_energy_model="fluid"):
        """model.py set_dark_energy: only the cosmological constant (w = -1, wa = 0) is part
        of this path, the reference's default; any other equation of state raises."""
        if w != -1.0 or wa != 0 or use_tabulated_w or dark_energy_model not in ("fluid", "ppf"):
            raise CAMBError("only a cosmological constant (w = -1, wa = 0) is part of the GPU path")
        return self

    def set_for_lmax(self, lmax, max_eta_k=None, lens_potential_accuracy=0, lens_output_margin=200,
                     k_eta_fac=2.5, lens_k_eta_reference=18000.0):
        """model.py:1018-1063 (the non-linear lensing switch is out of scope)."""
        self.max_l = lmax + lens_output_margin if self.DoLensing else lmax
        self.max_eta_k = max_eta_k or self.max_l * k_eta_fac
        if lens_potential_accuracy:
            self.max_eta_k = max(self.max_eta_k, lens_k_eta_reference * lens_potential_accuracy)
        return self

    def set_matter_power(self, redshifts=(0.0,), kmax=1.2, k_per_logint=None, nonlinear=None,
                         accurate_massive_neutrino_transfers=False, silent=False):
        """model.py:951-1016: transfer functions at the given redshifts to kmax (1/Mpc),
        high precision, optimized k spacing.  Non-linear corrections are out of scope."""
        if not len(redshifts):
            raise CAMBError("set_matter_power redshifts list is empty")
        if nonlinear:
            raise CAMBError("non-linear matter power is not part of the GPU path")
        if k_per_logint:
            raise CAMBError("only the optimized transfer k spacing (k_per_logint = 0) is built")
        if len(redshifts) > 256:
            raise CAMBError("at most 256 transfer redshifts (max_transfer_redshifts)")
        self.WantTransfer = True
        self.Transfer.high_precision = True
        self.Transfer.kmax = kmax
        self.Transfer.PK_redshifts = sorted(redshifts, reverse=True)
        return self

    def scalar_power(self, k):
        p = self.InitPower
        lnrat = math.log(k / p.pivot_scalar)
        return p.As * math.exp(lnrat * (p.ns - 1 + lnrat * (p.nrun / 2)))

    def to_struct(self):
        s = _lib.default_params()
        for n in ["H0", "ombh2", "omch2", "omk", "TCMB", "YHe", "nnu", "mnu", "num_massive_neutrinos", "Alens",
                  "max_l", "max_eta_k"]:
            setattr(s, n, getattr(self, n))
        s.max_l = int(self.max_l)
        s.optical_depth = self.Reion.optical_depth
        s.reion_delta_redshift = self.Reion.delta_redshift
        s.As, s.ns, s.nrun, s.pivot_scalar = (self.InitPower.As, self.InitPower.ns, self.InitPower.nrun,
                                              self.InitPower.pivot_scalar)
        s.do_lensing = 1 if self.DoLensing else 0
        for n in AccuracyParams._names:
            setattr(s, n, getattr(self.Accuracy, n))
        s.accurate_polarization = int(bool(self.Accuracy.AccuratePolarization))
        s.accurate_reionization = int(bool(self.Accuracy.AccurateReionization))
        s.want_cls = 1 if self.WantCls else 0
        s.want_transfer = 1 if self.WantTransfer else 0
        s.transfer_high_precision = 1 if self.Transfer.high_precision else 0
        s.transfer_kmax = self.Transfer.kmax
        zs = list(self.Transfer.PK_redshifts)
        s.num_transfer_redshifts = len(zs)
        for i, z in enumerate(zs):
            s.transfer_redshifts[i] = z
        s.reion_use_optical_depth = 1 if self.Reion.use_optical_depth else 0
        s.reion_redshift = self.Reion.redshift
        s.recfast_no_rosenbrock = 0 if self.Recomb.use_rosenbrock else 1
        return s


def set_params(cp=None, lmax=None, H0=None, ombh2=0.022, omch2=0.12, omk=0.0, mnu=0.06, nnu=3.044, YHe=None,
               tau=None, As=2e-9, ns=0.96, nrun=0, pivot_scalar=0.05, lens_potential_accuracy=0, max_eta_k=None,
               DoLensing=True, num_massive_neutrinos=1, **kwargs):
    """camb.set_params (camb.py:135) restricted to the parameters of the GPU scalar path."""
    cp = cp or CAMBparams()
    cp.DoLensing = DoLensing
    cp.set_cosmology(H0=H0 if H0 is not None else 67.5, ombh2=ombh2, omch2=omch2, omk=omk, mnu=mnu, nnu=nnu,
                     YHe=YHe, tau=tau, num_massive_neutrinos=num_massive_neutrinos)
    cp.InitPower.set_params(As=As, ns=ns, nrun=nrun, pivot_scalar=pivot_scalar)
    if lmax is not None:
        cp.set_for_lmax(lmax, max_eta_k=max_eta_k, lens_potential_accuracy=lens_potential_accuracy)
    # the remaining keywords as camb.set_params routes them (camb.py:200-238): the accuracy
    # and dark-energy setters, then attributes (dotted names reach sub-objects), and an
    # error for a name that is none of these
    de = {k: kwargs.pop(k) for k in ("w", "wa", "cs2", "use_tabulated_w", "wde_a_array", "wde_w_array",
                                     "dark_energy_model") if k in kwargs}
    if de:
        cp.set_dark_energy(**de)
    acc = {k: kwargs.pop(k) for k in ("AccuracyBoost", "lSampleBoost", "lAccuracyBoost", "DoLateRadTruncation",
                                      "min_l_logl_sampling") if k in kwargs}
    if acc:
        cp.set_accuracy(**{**dict(AccuracyBoost=cp.Accuracy.AccuracyBoost, lSampleBoost=cp.Accuracy.lSampleBoost,
                                  lAccuracyBoost=cp.Accuracy.lAccuracyBoost), **acc})
    for k, v in kwargs.items():
        obj, name = cp, k
        if "." in k:
            *path, name = k.split(".")
            for part in path:
                obj = getattr(obj, part)
        elif hasattr(cp.Accuracy, k):
            obj = cp.Accuracy
        if not hasattr(obj, name):
            raise CAMBError(f"Unrecognized parameter: {k}")
        setattr(obj, name, v)
    return cp
