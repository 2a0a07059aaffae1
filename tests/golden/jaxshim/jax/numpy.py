"""``jax.numpy`` stand-in: NumPy functions that drop sharding arguments and return JArray."""
import functools
import types
import numpy as _np

from ._core import JArray, asjarray

# dtype objects and classes pass straight through
integer = _np.integer
inexact = _np.inexact
floating = _np.floating
complexfloating = _np.complexfloating
finfo = _np.finfo
iinfo = _np.iinfo
issubdtype = _np.issubdtype
uint8 = _np.uint8
int32 = _np.int32
float64 = _np.float64
complex128 = _np.complex128
ndarray = JArray


def _wrap(fun):
    @functools.wraps(fun)
    def wrapper(*args, **kwargs):
        kwargs.pop('out_sharding', None)
        kwargs.pop('device', None)
        return asjarray(_to_array(fun(*args, **kwargs)))

    return wrapper


def _to_array(res):
    if isinstance(res, tuple):
        return tuple(_to_array(r) for r in res)
    if isinstance(res, _np.ndarray):
        return res
    if isinstance(res, _np.generic):
        return _np.asarray(res)
    return res


def bincount(x, weights=None, minlength=0, *, length=None):
    """jnp.bincount: with ``length``, values >= length are dropped and the output has that size."""
    x = _np.asarray(x)
    if length is None:
        return asjarray(_np.bincount(x, weights, minlength))
    keep = x < length
    w = None if weights is None else _np.asarray(weights)[keep]
    return asjarray(_np.bincount(x[keep], w, minlength=length)[:length])


def atan2(y, x):
    return asjarray(_np.asarray(_np.arctan2(y, x)))


linalg = types.SimpleNamespace(norm=_wrap(_np.linalg.norm), eigh=_wrap(_np.linalg.eigh))


def __getattr__(name):
    obj = getattr(_np, name)
    if callable(obj) and not isinstance(obj, type):
        return _wrap(obj)
    return obj
