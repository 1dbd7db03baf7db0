"""The array type of the stand-in: an ndarray with JAX's functional updates."""
import numpy as np


class JArray(np.ndarray):
    """ndarray with ``.at[idx].set/add/multiply/min/max/get`` returning new arrays."""

    def __array_finalize__(self, obj):
        pass

    @property
    def at(self):
        return _At(self)


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtRef(self._arr, idx)


class _AtRef:
    def __init__(self, arr, idx):
        self._arr = arr
        self._idx = idx

    def _copy(self):
        return np.array(self._arr, copy=True).view(JArray)

    def get(self, **_):
        return wrap(self._arr[self._idx])

    def set(self, v, **_):
        out = self._copy()
        out[self._idx] = np.asarray(v)
        return out

    def add(self, v, **_):
        out = self._copy()
        np.add.at(out, self._idx, np.asarray(v, dtype=out.dtype))
        return out

    def multiply(self, v, **_):
        out = self._copy()
        np.multiply.at(out, self._idx, np.asarray(v, dtype=out.dtype))
        return out

    def min(self, v, **_):
        out = self._copy()
        np.minimum.at(out, self._idx, np.asarray(v, dtype=out.dtype))
        return out

    def max(self, v, **_):
        out = self._copy()
        np.maximum.at(out, self._idx, np.asarray(v, dtype=out.dtype))
        return out


def wrap(x):
    """Arrays (and 0-d results) as JArray; Python objects unchanged."""
    if isinstance(x, JArray):
        return x
    if isinstance(x, np.ndarray):
        return x.view(JArray)
    if isinstance(x, np.generic):
        return np.asarray(x).view(JArray)
    return x


def tree_wrap(x):
    if isinstance(x, (list, tuple)) and not hasattr(x, "_fields"):
        return type(x)(tree_wrap(v) for v in x)
    return wrap(x)
