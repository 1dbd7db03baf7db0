"""The dispatcher operator torch.ops.astronomix_gb300.time_integration.

Its forward equals amx.time_integration on the same input; its gradient (the
discrete adjoint, recomputing the forward) equals the one of
time_integration_differentiable; its fake implementation gives the output's
shape and dtype without running.
"""
import numpy as np
import pytest

import astronomix_gb300 as amx
from astronomix_gb300 import torch_ops
from astronomix_gb300.adjoint import time_integration_differentiable

from _cases import smooth_random, rel_err

pytestmark = pytest.mark.gpu


def _case():
    return smooth_random(2, 16, seed=31, mhd=True, t_end=0.01, roll=True)


def test_operator_forward_equals_time_integration(cuda):
    import torch

    cfg, prm, rv, s = _case()
    key = torch_ops.register(cfg, prm, rv)
    out = torch_ops.ops().time_integration(torch.from_numpy(s.copy()).cuda(), key)
    ref = amx.time_integration(s.copy(), cfg, prm, rv)
    assert rel_err(out.cpu().numpy(), ref) < 1e-14


def test_operator_gradient_equals_adjoint(cuda):
    import torch

    cfg, prm, rv, s = _case()
    key = torch_ops.register(cfg, prm, rv)
    x = torch.from_numpy(s.copy()).cuda().requires_grad_()
    y = torch_ops.ops().time_integration(x, key)
    (y[0] ** 2).sum().backward()
    x2 = torch.from_numpy(s.copy()).cuda().requires_grad_()
    y2 = time_integration_differentiable(x2, cfg, prm, rv)
    (y2[0] ** 2).sum().backward()
    assert rel_err(x.grad.cpu().numpy(), x2.grad.cpu().numpy()) < 1e-12


def test_operator_fake_tensor_shapes():
    import torch
    from torch._subclasses.fake_tensor import FakeTensorMode

    cfg, prm, rv, s = _case()
    key = torch_ops.register(cfg, prm, rv)
    op = torch_ops.ops().time_integration
    with FakeTensorMode():
        x = torch.empty(s.shape, dtype=torch.float64)
        y = op(x, key)
    assert tuple(y.shape) == s.shape and y.dtype == torch.float64
