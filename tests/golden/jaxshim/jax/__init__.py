"""NumPy stand-in for the parts of jax that astronomix uses (test infrastructure)."""
import functools

import numpy as np

from . import _array
from ._array import JArray as Array


class _Config:
    jax_enable_x64 = True

    def update(self, name, value):
        setattr(self, name, value)


config = _Config()


def _static_decorator(fun=None, **_kw):
    if fun is None:
        return lambda f: f
    return fun


def _as_jax_args(v):
    """What jit does to its array arguments: NumPy arrays become jax arrays."""
    if isinstance(v, np.ndarray) and not isinstance(v, Array):
        return v.view(Array)
    if isinstance(v, (list, tuple)) and not hasattr(v, "_fields"):
        return type(v)(_as_jax_args(x) for x in v)
    return v


def jit(fun=None, **kw):
    """A plain call whose NumPy array arguments become jax arrays; no ``.lower``."""
    if fun is None:
        return lambda f: jit(f, **kw)

    @functools.wraps(fun)
    def called(*args, **kwargs):
        return fun(*[_as_jax_args(a) for a in args], **{k: _as_jax_args(v) for k, v in kwargs.items()})
    return called


def checkpoint(fun=None, **kw):
    return _static_decorator(fun, **kw)


remat = checkpoint


def vmap(fun, in_axes=0, out_axes=0):
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (list, tuple)) else [in_axes] * len(args)
        n = next(np.shape(a)[ax] for a, ax in zip(args, axes) if ax is not None)
        outs = [fun(*[a if ax is None else np.take(a, i, axis=ax) for a, ax in zip(args, axes)]) for i in range(n)]
        return _array.wrap(np.stack(outs, axis=out_axes))
    return mapped


def device_put(x, *_a, **_k):
    return x


def block_until_ready(x):
    return x


class NamedSharding:
    def __init__(self, *a, **k):
        self.args = a


class _Device:
    platform = "cpu"


def devices(*_a):
    return [_Device()]


from . import numpy, lax, random, debug, experimental, nn, tree_util  # noqa: E402,F401
