"""The time integration as PyTorch dispatcher operators.

``torch.ops.astronomix_gb300.time_integration(state, key)`` runs
``time_integration`` (astronomix/time_stepping/time_integration.py:61-236) on
a CUDA tensor and returns the final state as a new tensor; with autograd on a
finite-volume configuration its backward is the discrete adjoint (the
reference differentiates the same function with ``jax.grad``), which
recomputes the forward from the saved input (``time_integration_differentiable``
in adjoint.py keeps the forward's checkpoints instead).  The
reference marks ``config`` and ``registered_variables`` static (hashable
NamedTuples, time_integration.py:125-128); a dispatcher operator takes only
tensors and plain values, so the static arguments and the parameters are
registered once under a key (``register``) and the operator takes the key.

    key = register(config, params, registered_variables)
    out = torch.ops.astronomix_gb300.time_integration(state_cuda, key)

The operator has a fake (meta) implementation, so tracing tools see its
output shape and dtype without running it.
"""

import numpy as np

from .option_classes import SimulationConfig, SimulationParams, FINITE_VOLUME
from .variable_registry import RegisteredVariables

_REGISTRY = {}
_INTEGRATORS = {}
_OPS = None


def register(config: SimulationConfig, params: SimulationParams, registered_variables: RegisteredVariables) -> str:
    """The key under which the operator finds this configuration."""
    key = "amx%016x" % (hash((config, params, registered_variables)) & ((1 << 64) - 1))
    _REGISTRY[key] = (config, params, registered_variables)
    return key


def _lookup(key):
    try:
        return _REGISTRY[key]
    except KeyError:
        raise KeyError("configuration %r was not registered with astronomix_gb300.torch_ops.register" % key)


def _integrator(key, state):
    from .adjoint import AdjointIntegrator

    config, params, rv = _lookup(key)
    dtype = np.float64 if state.dtype.is_floating_point and state.element_size() == 8 else np.float32
    ik = (key, tuple(state.shape), dtype)
    integ = _INTEGRATORS.get(ik)
    if integ is None:
        integ = AdjointIntegrator(config, params, rv, tuple(state.shape), dtype, tape_budget="auto")
        _INTEGRATORS[ik] = integ
    return integ


def ops():
    """Registers the operators (once) and returns torch.ops.astronomix_gb300."""
    global _OPS
    if _OPS is not None:
        return _OPS
    import torch

    @torch.library.custom_op("astronomix_gb300::time_integration", mutates_args=())
    def time_integration_op(state: torch.Tensor, key: str) -> torch.Tensor:
        from .time_integration import time_integration

        config, params, rv = _lookup(key)
        if not state.is_cuda:
            raise ValueError("astronomix_gb300::time_integration takes a CUDA tensor")
        return time_integration(state.detach(), config, params, rv)

    @time_integration_op.register_fake
    def _(state, key):
        return torch.empty_like(state)

    # the backward keeps no state from the forward: it recomputes the forward
    # from the saved input through the adjoint integrator (which records the
    # dt schedule and checkpoints) and pulls the cotangent back through it
    def setup_context(ctx, inputs, output):
        ctx.key = inputs[1]
        ctx.save_for_backward(inputs[0])

    def backward(ctx, grad):
        config, _, _ = _lookup(ctx.key)
        if config.solver_mode != FINITE_VOLUME:
            raise NotImplementedError("the discrete adjoint covers the finite-volume scheme")
        (x,) = ctx.saved_tensors
        integ = _integrator(ctx.key, x)
        integ.forward(x.detach())
        return integ.backward(grad.contiguous()), None

    torch.library.register_autograd("astronomix_gb300::time_integration", backward, setup_context=setup_context)
    _OPS = torch.ops.astronomix_gb300
    return _OPS
