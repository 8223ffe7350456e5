"""Host logic of the finite-difference gradients: the batch members and their steps."""
import numpy as np

from camb_gb300 import gradients, model


def test_members_perturb_one_parameter_each():
    ps = [model.set_params(lmax=600, DoLensing=False, mnu=0.0, tau=0.055, H0=68.0),
          model.set_params(lmax=600, DoLensing=False, mnu=0.1, tau=0.06, ombh2=0.0225)]
    members, steps = gradients.fd_members(ps, 1e-4)
    stride = 1 + 2 * len(gradients.EVOLVED)
    assert len(members) == stride * len(ps)
    for i, p in enumerate(ps):
        assert members[i * stride] is p
        for j, name in enumerate(gradients.EVOLVED):
            v = gradients.get_param(p, name)
            h = steps[i][j]
            assert np.isclose(h, 1e-4 * abs(v))
            plus, minus = members[i * stride + 1 + 2 * j], members[i * stride + 2 + 2 * j]
            assert gradients.get_param(plus, name) == v + h
            assert gradients.get_param(minus, name) == v - h
            for other in gradients.PARAMS:
                if other != name:
                    assert gradients.get_param(plus, other) == gradients.get_param(p, other)
                    assert gradients.get_param(minus, other) == gradients.get_param(p, other)
    # the inputs themselves are untouched
    assert ps[0].H0 == 68.0 and ps[1].ombh2 == 0.0225
