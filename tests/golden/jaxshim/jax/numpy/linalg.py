import numpy as _np

from .._array import wrap


def norm(x, ord=None, axis=None, keepdims=False):  # noqa: A002
    """jnp.linalg.norm's vector 2-norm: sqrt(sum(|x|^2)) along the axis."""
    x = _np.asarray(x)
    if ord in (None, 2) and axis is not None and not isinstance(axis, tuple):
        return wrap(_np.sqrt(_np.sum(_np.real(x * _np.conj(x)), axis=axis, keepdims=keepdims)))
    return wrap(_np.linalg.norm(x, ord=ord, axis=axis, keepdims=keepdims))
