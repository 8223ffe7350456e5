"""Finite-difference gradients through the batched GPU pipeline: dC_l/dAs against the
exact C_l/As at the sampled l (between them InterpolateCls splines the difference from
the fixed high-L template, so the interpolated C_l are affine, not proportional, in As),
dC_l/dns against a tenfold step, and dC_l/d(ombh2, tau) against central
differences of the oracle's C_l for the same perturbed cosmologies (agreement 1e-3 of
each gradient's peak over l); the autograd wrapper contracts the same Jacobian.  At the
gradient configuration's size: all four evolved parameters on two massive-neutrino draws of
its box at lmax 2500 against the oracle's differences, and the finite-difference noise
stated as the agreement of two relative steps."""
import copy

import numpy as np
import pytest

from camb_gb300 import _lib, gradients, model
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def base(lmax=600, mnu=0.0):
    return model.set_params(lmax=lmax, DoLensing=False, mnu=mnu, tau=0.06, H0=67.5, ombh2=0.022, omch2=0.122,
                            As=2.1e-9, ns=0.965)


@pytest.fixture(scope="module")
def grads():
    ps = [base(), base(mnu=0.1)]
    cls, g = gradients.cl_gradients(ps)
    return ps, cls, g


def test_as_and_ns(grads):
    ps, cls, g = grads
    l = np.arange(2, 601)
    for i, p in enumerate(ps):
        ls = _lib.Tables(p.to_struct()).ls
        dAs = g[i, gradients.PARAMS.index("As")]
        np.testing.assert_allclose(dAs[ls, :2], cls[i][ls, :2] / p.InitPower.As, rtol=1e-7)
    _, g10 = gradients.cl_gradients([ps[0]], rel_step=1e-3)
    j = gradients.PARAMS.index("ns")
    peak = np.max(np.abs(g[0, j][l, 0]))
    assert np.max(np.abs(g10[0, j][l, 0] - g[0, j][l, 0])) / peak < 1e-5


@pytest.mark.parametrize("name", ["ombh2", "tau"])
def test_evolved_parameters_match_oracle_differences(grads, name):
    ps, _, g = grads
    p = ps[0]
    j = gradients.PARAMS.index(name)
    v = gradients.get_param(p, name)
    h = 1e-4 * abs(v)
    icl = []
    for sgn in (1.0, -1.0):
        q = model.set_params(lmax=600, DoLensing=False, mnu=0.0, tau=0.06, H0=67.5, ombh2=0.022, omch2=0.122,
                             As=2.1e-9, ns=0.965)
        gradients.set_param(q, name, v + sgn * h)
        T = _lib.Tables(q.to_struct())
        icl.append(orc.cls(T, orc.los(T, orc.evolve_sources(T))))
        ls = T.ls
    ref = (icl[0] - icl[1]) / (2 * h)
    got = g[0, j][ls]
    for c_got, c_ref in [(0, 0), (1, 1)]:
        peak = np.max(np.abs(ref[:, c_ref]))
        assert np.max(np.abs(got[:, c_got] - ref[:, c_ref])) / peak < 1e-3


def test_autograd_contracts_the_jacobian(grads):
    torch = pytest.importorskip("torch")
    ps, cls, g = grads
    f = gradients.cls_function()
    theta = torch.tensor([[gradients.get_param(ps[0], n) for n in gradients.PARAMS]], dtype=torch.float64,
                         requires_grad=True)
    out = f.apply(theta, ps[0])
    w = torch.zeros_like(out)
    w[0, 2:, 0] = 1.0
    (out * w).sum().backward()
    want = g[0][:, 2:, 0].sum(axis=1)
    np.testing.assert_allclose(theta.grad.numpy()[0], want, rtol=1e-6)


def box_draws(n, seed=3000, lmax=2500):
    """Draws of the gradient configuration's box, as the benchmark makes them: each of
    ombh2, omch2, H0, tau, As, ns uniform in fiducial +-5%, mnu uniform in [0, 0.2] eV."""
    rng = np.random.default_rng(seed)
    ps = []
    for _ in range(n):
        f = lambda v: v * (1 + 0.05 * (2 * rng.random() - 1))  # noqa: E731
        ps.append(model.set_params(lmax=lmax, DoLensing=False, H0=f(67.5), ombh2=f(0.022), omch2=f(0.122),
                                   tau=f(0.06), As=f(2.1e-9), ns=f(0.965), mnu=0.2 * rng.random(), nnu=3.046))
    return ps


@pytest.fixture(scope="module")
def box():
    ps = box_draws(2)
    assert all(p.to_struct().mnu > 0 for p in ps)
    _, g = gradients.cl_gradients(ps)
    return ps, g


def oracle_fd(p, name, rel_step=1e-4):
    v = gradients.get_param(p, name)
    h = rel_step * abs(v)
    icl = []
    for sgn in (1.0, -1.0):
        q = copy.deepcopy(p)
        gradients.set_param(q, name, v + sgn * h)
        T = _lib.Tables(q.to_struct())
        icl.append(orc.cls(T, orc.los(T, orc.evolve_sources(T))))
    return T.ls, (icl[0] - icl[1]) / (2 * h)


@pytest.mark.parametrize("name", gradients.EVOLVED)
def test_box_gradients_match_oracle_differences(box, name):
    """dC_l/d(ombh2, omch2, H0, tau) on two massive-neutrino draws of the gradient box at
    lmax 2500: the batched GPU central differences against the oracle's central
    differences of the same perturbed cosmologies, within 1e-3 of each gradient's peak over
    the sampled l, for TT, EE and TE.  Both sides make the same step decisions, so their
    agreement does not depend on the finite-difference noise stated below."""
    ps, g = box
    j = gradients.PARAMS.index(name)
    for i, p in enumerate(ps):
        ls, ref = oracle_fd(p, name)
        got = g[i, j][ls]
        for c_got, c_ref in [(0, 0), (1, 1), (3, 2)]:
            peak = np.max(np.abs(ref[:, c_ref]))
            assert np.max(np.abs(got[:, c_got] - ref[:, c_ref])) / peak < 1e-3, (i, name, c_got)


def test_fd_noise_between_relative_steps(box):
    """The finite-difference noise of the gradients, stated as the agreement of relative
    steps 1e-4 and 3e-4 on the same two draws (sampled l, relative to each gradient's peak
    over l).  Both steps sit near the ODE tolerance (1e-4), where an accept/reject decision
    of the adaptive stepper that flips between the + and - members moves C_l by a few
    1e-6 and the difference quotient by up to the gradient itself at single l (the grids of
    the two members have identical sizes, so the noise is not a grid jump).  Measured on
    the oracle for these draws: EE within 3e-3 of its peak everywhere; TT and TE within
    5e-3 at the median l, within 0.1 at 90% of the l, and up to 0.8 (TT) at a few l of
    the draw with the lightest neutrino."""
    ps, g = box
    _, g3 = gradients.cl_gradients(ps, rel_step=3e-4)
    for i, p in enumerate(ps):
        ls = _lib.Tables(p.to_struct()).ls
        ls = ls[ls >= 2]
        for name in gradients.EVOLVED:
            j = gradients.PARAMS.index(name)
            for c in (0, 1, 3):
                a, b = g[i, j][ls, c], g3[i, j][ls, c]
                d = np.abs(a - b) / np.max(np.abs(a))
                if c == 1:
                    assert d.max() < 5e-3, (i, name, "EE", d.max())
                else:
                    assert np.median(d) < 5e-3, (i, name, c, np.median(d))
                    assert np.quantile(d, 0.9) < 0.15, (i, name, c, np.quantile(d, 0.9))


def test_gradients_use_the_fp64_projection_whatever_the_callers_setting(grads):
    """cl_gradients runs its batch with the FP64 projection by default, so a caller that
    left the mixed projection set gets the FP64 gradients (the mixed projection would move
    them by ~1e-3 of their peak), and keeps its setting."""
    ps, cls, g = grads
    lib = _lib.load()
    old = lib.cambgpu_get_precision()
    _lib.check(lib.cambgpu_set_precision(1))
    try:
        cls1, g1 = gradients.cl_gradients(ps)
        assert lib.cambgpu_get_precision() == 1
    finally:
        lib.cambgpu_set_precision(old)
    np.testing.assert_allclose(cls1, cls, rtol=1e-12, atol=0)
    for j in range(len(gradients.PARAMS)):
        for c in (0, 1, 3):
            peak = np.max(np.abs(g[:, j, 2:, c]))
            assert np.max(np.abs(g1[:, j, 2:, c] - g[:, j, 2:, c])) < 1e-9 * peak
