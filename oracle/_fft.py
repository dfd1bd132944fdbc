"""FFT backend of the oracle: scipy.fft (pocketfft) with a configurable number
of worker threads (``set_workers``); numpy.fft semantics (MATLAB fft/fftn/ifftn
sign and 1/n conventions)."""
import os

import scipy.fft as _sf

_WORKERS = 1


def set_workers(n=None):
    global _WORKERS
    _WORKERS = int(n or os.cpu_count() or 1)
    return _WORKERS


def workers():
    return _WORKERS


def fft(a, axis=-1):
    return _sf.fft(a, axis=axis, workers=_WORKERS)


def ifft(a, axis=-1):
    return _sf.ifft(a, axis=axis, workers=_WORKERS)


def fftn(a, s=None, axes=None):
    return _sf.fftn(a, s=s, axes=axes, workers=_WORKERS)


def ifftn(a, axes=None):
    return _sf.ifftn(a, axes=axes, workers=_WORKERS)
