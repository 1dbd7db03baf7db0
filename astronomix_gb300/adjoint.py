"""Reverse-mode gradients of the FV time integration (hand-written discrete adjoint).

The reference differentiates ``time_integration`` with ``jax.grad``
(tests/mhd_tests/mhd_correct.py:237-264): the adaptive dt is held fixed
(``stop_gradient``, astronomix/time_stepping/time_integration.py:632-661) and
the magnetic fixed point is differentiated through the iterations it took.
Here the same gradient comes from the C ABI's adjoint (include/amx.h,
amx_adjoint_*): the forward runs the ordinary GPU step, keeping a checkpoint
every ``checkpoint_every`` steps; the backward replays one segment at a time
and applies the hand-derived vector-Jacobian products of every stage in
reverse.  ``time_integration_differentiable`` wraps it in a
``torch.autograd.Function``, so ``loss.backward()`` works as ``jax.grad`` does
on the reference.
"""

import numpy as np

from . import _native
from .option_classes import SimulationConfig, SimulationParams, FINITE_VOLUME
from .time_integration import make_amx_config, _check_supported, _stream, _raise_status
from .variable_registry import RegisteredVariables

__all__ = ["AdjointIntegrator", "time_integration_differentiable"]


class AdjointIntegrator:
    """Forward / backward / replay of one FV configuration on the GPU.

    ``forward(x)`` returns the final state (a new CUDA tensor) and records the
    schedule; ``backward(g)`` returns d<g, final>/d(initial state) for the last
    forward; ``replay(x)`` integrates ``x`` with the recorded schedule (fixed
    dt and iteration counts), the program the gradient is exact for.
    """

    def __init__(self, config: SimulationConfig, params: SimulationParams, registered_variables: RegisteredVariables,
                 shape, dtype=np.float32, checkpoint_every=20, max_steps=1 << 20):
        _check_supported(config)
        if config.solver_mode != FINITE_VOLUME:
            raise NotImplementedError("the adjoint covers the finite-volume scheme")
        self.config = config
        self.params = params
        self.rv = registered_variables
        self.shape = tuple(shape)
        self.dtype = np.dtype(dtype)
        self.checkpoint_every = int(checkpoint_every)
        self.prm = _native.make_params(params)
        self.adj = _native.Adjoint(make_amx_config(config, registered_variables, shape, self.dtype),
                                   self.checkpoint_every, max_steps)
        self.info = None

    def _check(self, x):
        import torch

        want = torch.float64 if self.dtype == np.float64 else torch.float32
        if not (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == want and tuple(x.shape) == self.shape):
            raise ValueError("expected a CUDA tensor of shape %s and dtype %s" % (self.shape, want))
        return x.detach().contiguous()

    def forward(self, x):
        y = self._check(x).clone()
        self.info = self.adj.forward(y.data_ptr(), self.prm, _stream())
        _raise_status(self.info.status, self.config)
        return y

    def backward(self, grad_final):
        import torch

        g = self._check(grad_final)
        out = torch.empty_like(g)
        self.adj.backward(g.data_ptr(), out.data_ptr(), _stream())
        return out

    def replay(self, x):
        y = self._check(x).clone()
        self.adj.replay(y.data_ptr(), _stream())
        return y

    def schedule(self):
        """(dt per step, fixed-point iterations per step) of the last forward."""
        return self.adj.schedule()

    def memory(self):
        return self.adj.memory()


def _function():
    import torch

    class _TimeIntegration(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, integrator):
            ctx.integrator = integrator
            return integrator.forward(x)

        @staticmethod
        def backward(ctx, grad):
            return ctx.integrator.backward(grad.contiguous()), None

    return _TimeIntegration


_FN = None


def time_integration_differentiable(primitive_state, config: SimulationConfig, params: SimulationParams,
                                    registered_variables: RegisteredVariables, checkpoint_every=20,
                                    integrator=None):
    """``time_integration`` as a differentiable torch op on a CUDA tensor:
    the result's gradient flows back to ``primitive_state`` through the
    discrete adjoint.  Pass an ``AdjointIntegrator`` to reuse its buffers."""
    global _FN
    if _FN is None:
        _FN = _function()
    if integrator is None:
        integrator = AdjointIntegrator(config, params, registered_variables, tuple(primitive_state.shape),
                                       np.float64 if str(primitive_state.dtype) == "torch.float64" else np.float32,
                                       checkpoint_every)
    return _FN.apply(primitive_state, integrator)
