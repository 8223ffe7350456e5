"""Finite-difference gradients through the batched GPU pipeline: dC_l/dAs against the
exact C_l/As at the sampled l (between them InterpolateCls splines the difference from
the fixed high-L template, so the interpolated C_l are affine, not proportional, in As),
dC_l/dns against a tenfold step, and dC_l/d(ombh2, tau) against central
differences of the oracle's C_l for the same perturbed cosmologies (agreement 1e-3 of
each gradient's peak over l); the autograd wrapper contracts the same Jacobian."""
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
