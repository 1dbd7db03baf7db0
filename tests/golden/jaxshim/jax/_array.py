"""The array type of the stand-in: an ndarray with JAX's functional updates."""
import numpy as np


def _static_ints(arr, idx):
    """The index as a tuple, and whether one of its static integer entries
    (before any Ellipsis, None or array entry) lies outside its axis."""
    t = idx if isinstance(idx, tuple) else (idx,)
    out = False
    for ax, e in enumerate(t):
        if e is Ellipsis or e is None or isinstance(e, (np.ndarray, list)):
            break
        if isinstance(e, (int, np.integer)) and not isinstance(e, bool) and ax < arr.ndim:
            if not -arr.shape[ax] <= int(e) < arr.shape[ax]:
                out = True
    return t, out


def _clamped(arr, t):
    """JAX's retrieval semantics: static out-of-range integers clamp to the
    axis (jax.numpy indexing gathers with clamped indices)."""
    r = []
    for ax, e in enumerate(t):
        if isinstance(e, (int, np.integer)) and not isinstance(e, bool) and ax < arr.ndim:
            n = arr.shape[ax]
            e = int(e)
            e = e + n if -n <= e < 0 else e
            e = min(max(e, 0), n - 1)
        r.append(e)
    return tuple(r)


class JArray(np.ndarray):
    """ndarray with ``.at[idx].set/add/multiply/min/max/get`` returning new
    arrays, and JAX's handling of static integer indices outside an axis:
    reads clamp them, updates through ``.at`` are dropped (NumPy would raise
    IndexError for both)."""

    def __array_finalize__(self, obj):
        pass

    def __getitem__(self, idx):
        t, out = _static_ints(self, idx)
        if out:
            idx = _clamped(self, t)
        return super().__getitem__(idx)

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

    def _dropped(self):
        # an update at a static index outside its axis is dropped (JAX)
        return _static_ints(self._arr, self._idx)[1]

    def get(self, **_):
        return wrap(self._arr[self._idx])

    def set(self, v, **_):
        out = self._copy()
        if self._dropped():
            return out
        out[self._idx] = np.asarray(v)
        return out

    def add(self, v, **_):
        out = self._copy()
        if self._dropped():
            return out
        np.add.at(out, self._idx, np.asarray(v, dtype=out.dtype))
        return out

    def multiply(self, v, **_):
        out = self._copy()
        if self._dropped():
            return out
        np.multiply.at(out, self._idx, np.asarray(v, dtype=out.dtype))
        return out

    def min(self, v, **_):
        out = self._copy()
        if self._dropped():
            return out
        np.minimum.at(out, self._idx, np.asarray(v, dtype=out.dtype))
        return out

    def max(self, v, **_):
        out = self._copy()
        if self._dropped():
            return out
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
