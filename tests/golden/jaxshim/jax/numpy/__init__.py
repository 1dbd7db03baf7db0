"""jax.numpy on NumPy: every function returns JArray views (test infrastructure)."""
import functools

import numpy as _np

from .._array import JArray, wrap, tree_wrap

ndarray = _np.ndarray
pi = _np.pi
e = _np.e
inf = _np.inf
nan = _np.nan
newaxis = None
float32, float64, int32, int64, bool_, complex64, complex128 = (
    _np.float32, _np.float64, _np.int32, _np.int64, _np.bool_, _np.complex64, _np.complex128)
int = _np.int64  # noqa: A001
float = _np.float64  # noqa: A001
uint32 = _np.uint32
dtype = _np.dtype
finfo = _np.finfo
iinfo = _np.iinfo


def _wrapped(f):
    @functools.wraps(f)
    def g(*a, **k):
        return tree_wrap(f(*a, **k))
    return g


def array(x, dtype=None, copy=True, **_):
    return wrap(_np.array(x, dtype=dtype))


def asarray(x, dtype=None, **_):
    return wrap(_np.asarray(x, dtype=dtype))


def einsum(*a, **k):
    k.pop("precision", None)
    k.pop("preferred_element_type", None)
    return wrap(_np.einsum(*a, **k))


def vectorize(pyfunc=None, **kw):
    if pyfunc is None:
        return lambda f: vectorize(f, **kw)
    kw.pop("excluded", None)
    return _wrapped(_np.vectorize(pyfunc, **kw))


_cache = {}


def __getattr__(name):
    if name in _cache:
        return _cache[name]
    f = getattr(_np, name)
    if callable(f) and not isinstance(f, type):
        f = _wrapped(f)
    _cache[name] = f
    return f


from . import fft, linalg  # noqa: E402,F401
