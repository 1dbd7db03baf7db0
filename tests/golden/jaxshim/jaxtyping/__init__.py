"""Type annotations of jaxtyping as inert placeholders."""
from typing import Any


class _Sub:
    def __class_getitem__(cls, item):
        return Any


class Float(_Sub):
    pass


class Int(_Sub):
    pass


class Bool(_Sub):
    pass


class Shaped(_Sub):
    pass


Array = Any
PyTree = Any
PRNGKeyArray = Any
ArrayLike = Any
Key = Any


def jaxtyped(fun=None, *, typechecker=None):
    if fun is None:
        return lambda f: f
    return fun
