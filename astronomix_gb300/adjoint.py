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

__all__ = ["AdjointIntegrator", "time_integration_differentiable", "density_perturbation_problem"]


class AdjointIntegrator:
    """Forward / backward / replay of one FV configuration on the GPU.

    ``forward(x)`` returns the final state (a new CUDA tensor) and records the
    schedule; ``backward(g)`` returns d<g, final>/d(initial state) for the last
    forward; ``replay(x)`` integrates ``x`` with the recorded schedule (fixed
    dt and iteration counts), the program the gradient is exact for.

    ``tape_budget`` (bytes, or ``"auto"`` for half the free device memory)
    lets the forward store the whole tape when it fits, so that the backward
    recomputes nothing; with 0, or when the run does not fit, the forward
    keeps a checkpoint every ``checkpoint_every`` steps and the backward
    replays one segment at a time.
    """

    def __init__(self, config: SimulationConfig, params: SimulationParams, registered_variables: RegisteredVariables,
                 shape, dtype=np.float32, checkpoint_every=20, max_steps=1 << 20, tape_budget=0):
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
        if tape_budget == "auto":
            import torch

            tape_budget = int(torch.cuda.mem_get_info()[0] * 0.5)
        self.adj.set_tape_budget(int(tape_budget))
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

    def stored_tape(self) -> bool:
        """Whether the last forward stored the whole tape (no recompute)."""
        return self.adj.uses_stored_tape()

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
                                    integrator=None, tape_budget="auto"):
    """``time_integration`` as a differentiable torch op on a CUDA tensor:
    the result's gradient flows back to ``primitive_state`` through the
    discrete adjoint.  Pass an ``AdjointIntegrator`` to reuse its buffers."""
    global _FN
    if _FN is None:
        _FN = _function()
    if integrator is None:
        integrator = AdjointIntegrator(config, params, registered_variables, tuple(primitive_state.shape),
                                       np.float64 if str(primitive_state.dtype) == "torch.float64" else np.float32,
                                       checkpoint_every, tape_budget=tape_budget)
    return _FN.apply(primitive_state, integrator)


def density_perturbation_problem(n=128, seed=0, target_seed=1, amplitude=0.1, t_end=0.1, C_cfl=0.25,
                                 dtype=np.float32):
    """The inverse-problem benchmark of the adjoint: 3D ideal MHD on the
    periodic unit cube, FV HLL + the Pang-Wu magnetic split, MINMOD, gamma
    5/3; rho = 1 + amplitude * g with g a 3D Gaussian random field of per-mode
    power ~ k^-3 (amplitude slope -1.5, 1 <= k <= 0.7 n / 2) scaled to unit
    standard deviation, p = 1, v = 0, uniform B_z = 1 (plasma beta 2), to
    t_end.  The target density comes from the same recipe with
    ``target_seed``.  Returns (config, params, registered_variables, state,
    target_density)."""
    from .ensemble import create_turb_field
    from .option_classes import (BoundarySettings, BoundarySettings1D, PERIODIC_BOUNDARY, HLL, MINMOD,
                                 SINGLE_PRECISION, DOUBLE_PRECISION, finalize_config)
    from .setup_helpers import construct_primitive_state
    from .variable_registry import get_registered_variables

    def field(sd):
        g = create_turb_field(n, 1.0, -1.5, 1.0, 0.7 * n / 2, seed=sd, dimensionality=3)
        return 1.0 + amplitude * g / g.std()

    cfg = SimulationConfig(
        mhd=True, dimensionality=3, box_size=1.0, num_cells=n, riemann_solver=HLL, limiter=MINMOD,
        numerical_precision=DOUBLE_PRECISION if np.dtype(dtype) == np.float64 else SINGLE_PRECISION,
        boundary_settings=BoundarySettings(*[BoundarySettings1D(PERIODIC_BOUNDARY, PERIODIC_BOUNDARY)] * 3))
    rv = get_registered_variables(cfg)
    rho = field(seed)
    z = np.zeros_like(rho)
    state = construct_primitive_state(cfg, rv, density=rho.astype(dtype), velocity_x=z, velocity_y=z,
                                      velocity_z=z, gas_pressure=np.ones_like(rho), magnetic_field_x=z,
                                      magnetic_field_y=z, magnetic_field_z=np.ones_like(rho))
    cfg = finalize_config(cfg, state.shape)
    prm = SimulationParams(t_end=t_end, gamma=5.0 / 3.0, C_cfl=C_cfl)
    return cfg, prm, rv, state, field(target_seed).astype(dtype)
