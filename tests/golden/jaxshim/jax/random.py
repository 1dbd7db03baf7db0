"""Seeded NumPy generators in place of jax.random (the values are not threefry's)."""
import numpy as np

from ._array import wrap


class _Key:
    def __init__(self, seed):
        self.seed = np.random.SeedSequence(seed)


def key(seed):
    return _Key(int(seed))


PRNGKey = key


def split(k, num=2):
    out = []
    for child in k.seed.spawn(num):
        kk = _Key(0)
        kk.seed = child
        out.append(kk)
    return out


def normal(k, shape=(), dtype=np.float64):
    return wrap(np.random.default_rng(k.seed).standard_normal(shape).astype(dtype))


def uniform(k, shape=(), dtype=np.float64, minval=0.0, maxval=1.0):
    return wrap(np.random.default_rng(k.seed).uniform(minval, maxval, shape).astype(dtype))
