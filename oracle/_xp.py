"""Array-namespace shim for the oracle (test infrastructure only).

The oracle restates the reference's JAX code operation for operation.  It runs
on NumPy for value parity and on torch (CPU, float64) when a test needs
reverse-mode gradients, the stand-in for ``jax.grad`` of the reference.  Both
backends expose the handful of primitives the restatement uses, with the
reference's semantics: ``roll`` wraps like ``jnp.roll``, ``sign(0) == 0``,
``maximum``/``minimum`` are elementwise and accept Python scalars.
"""

import numpy as np


class _NumpyBackend:
    name = "numpy"

    @staticmethod
    def roll(a, shift, axis):
        return np.roll(a, shift, axis=axis)

    where = staticmethod(np.where)
    sqrt = staticmethod(np.sqrt)
    abs = staticmethod(np.abs)
    sign = staticmethod(np.sign)
    sin = staticmethod(np.sin)

    @staticmethod
    def maximum(a, b):
        return np.maximum(a, b)

    @staticmethod
    def minimum(a, b):
        return np.minimum(a, b)

    @staticmethod
    def zeros_like(a):
        return np.zeros_like(a)

    @staticmethod
    def copy(a):
        return np.array(a, copy=True)

    @staticmethod
    def stack(arrs, axis=0):
        return np.stack(arrs, axis=axis)

    @staticmethod
    def concatenate(arrs, axis=0):
        return np.concatenate(arrs, axis=axis)

    @staticmethod
    def amax(a):
        return np.max(a)

    @staticmethod
    def transpose(a, perm):
        return np.transpose(a, perm)

    @staticmethod
    def pad_edge(a, width, dims):
        pads = ((0, 0),) + ((width, width),) * dims
        return np.pad(a, pads, mode="edge")

    @staticmethod
    def scalar(value, like):
        return np.asarray(value, dtype=like.dtype)

    @staticmethod
    def to_float(x):
        return float(x)


class _TorchBackend:
    name = "torch"

    def __init__(self):
        import torch

        self.t = torch

    def roll(self, a, shift, axis):
        return self.t.roll(a, shifts=shift, dims=axis)

    def _as(self, x, like):
        if isinstance(x, self.t.Tensor):
            return x
        return self.t.as_tensor(x, dtype=like.dtype)

    def where(self, c, a, b):
        ref = a if isinstance(a, self.t.Tensor) else b
        return self.t.where(c, self._as(a, ref), self._as(b, ref))

    def sqrt(self, a):
        return self.t.sqrt(a)

    def abs(self, a):
        return self.t.abs(a)

    def sign(self, a):
        return self.t.sign(a)

    def sin(self, a):
        return self.t.sin(a)

    def maximum(self, a, b):
        ref = a if isinstance(a, self.t.Tensor) else b
        return self.t.maximum(self._as(a, ref), self._as(b, ref))

    def minimum(self, a, b):
        ref = a if isinstance(a, self.t.Tensor) else b
        return self.t.minimum(self._as(a, ref), self._as(b, ref))

    def zeros_like(self, a):
        return self.t.zeros_like(a)

    def copy(self, a):
        return a.clone()

    def stack(self, arrs, axis=0):
        return self.t.stack(list(arrs), dim=axis)

    def concatenate(self, arrs, axis=0):
        return self.t.cat(list(arrs), dim=axis)

    def amax(self, a):
        return self.t.max(a)

    def transpose(self, a, perm):
        return a.permute(*perm)

    def pad_edge(self, a, width, dims):
        # edge padding along the trailing `dims` spatial axes
        out = a
        for ax in range(1, dims + 1):
            n = out.shape[ax]
            left = out.narrow(ax, 0, 1).expand(*[width if i == ax else s for i, s in enumerate(out.shape)])
            right = out.narrow(ax, n - 1, 1).expand(*[width if i == ax else s for i, s in enumerate(out.shape)])
            out = self.t.cat([left, out, right], dim=ax)
        return out

    def scalar(self, value, like):
        return self.t.as_tensor(value, dtype=like.dtype)

    def to_float(self, x):
        return float(x.detach()) if hasattr(x, "detach") else float(x)


class _Proxy:
    """Forwards attribute access to the active backend."""

    def __init__(self):
        self._impl = _NumpyBackend()

    def __getattr__(self, item):
        return getattr(self._impl, item)


xp = _Proxy()


def set_backend(name: str) -> None:
    """Select ``"numpy"`` (default) or ``"torch"`` for all oracle functions."""
    if name == "numpy":
        xp._impl = _NumpyBackend()
    elif name == "torch":
        xp._impl = _TorchBackend()
    else:
        raise ValueError(name)


class backend:
    """Context manager: ``with backend("torch"): ...``."""

    def __init__(self, name):
        self.name = name

    def __enter__(self):
        self.prev = xp._impl.name
        set_backend(self.name)

    def __exit__(self, *exc):
        set_backend(self.prev)
