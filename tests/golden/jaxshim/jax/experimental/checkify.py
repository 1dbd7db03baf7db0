"""checkify: checks raise at once; checkify(f) returns (error, result)."""
import numpy as np


class JaxRuntimeError(RuntimeError):
    pass


class _ErrSet(frozenset):
    def __or__(self, other):
        return _ErrSet(frozenset.__or__(self, other))


user_checks = _ErrSet({"user"})
index_checks = _ErrSet({"index"})
float_checks = _ErrSet({"float"})
nan_checks = _ErrSet({"nan"})
div_checks = _ErrSet({"div"})
all_checks = user_checks | index_checks | float_checks | nan_checks | div_checks


def check(pred, msg, *fmt_args, **fmt_kwargs):
    if not bool(np.all(pred)):
        raise JaxRuntimeError(msg.format(*fmt_args, **fmt_kwargs))


class _NoError:
    def throw(self):
        return None

    def get(self):
        return None


def checkify(fun, errors=user_checks):
    def checked(*a, **k):
        return _NoError(), fun(*a, **k)
    return checked
