"""jax.numpy -> NumPy."""
import numpy as _np
from numpy import *  # noqa: F401,F403
from numpy import linalg  # noqa: F401

ndarray = _np.ndarray
pi = _np.pi
newaxis = None


def asarray(a, dtype=None, **k):
    return _np.asarray(a, dtype=dtype)


def array(a, dtype=None, **k):
    return _np.array(a, dtype=dtype)
