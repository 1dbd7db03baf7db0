from .units import _Quantity


def __getattr__(name):
    return _Quantity()
