"""equinox stand-in: Module as a plain base class, filters and nn as stubs."""
from . import nn, internal  # noqa: F401


class Module:
    pass


def combine(*trees):
    for t in trees:
        if t is not None:
            return t
    return None


def partition(tree, *_a, **_k):
    return tree, None


def filter_jit(fun=None, **_):
    return fun if fun is not None else (lambda f: f)


def is_array(x):
    import numpy as np
    return isinstance(x, np.ndarray)
