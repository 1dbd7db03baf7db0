import numpy as _np

from .._array import wrap


def _w(name):
    f = getattr(_np.fft, name)

    def g(*a, **k):
        return wrap(f(*a, **k))
    g.__name__ = name
    return g


fftn, ifftn, rfftn, irfftn, fft, ifft, rfft, irfft, fftfreq, rfftfreq, fftshift, ifftshift = (
    _w(n) for n in ("fftn", "ifftn", "rfftn", "irfftn", "fft", "ifft", "rfft", "irfft", "fftfreq", "rfftfreq",
                    "fftshift", "ifftshift"))
